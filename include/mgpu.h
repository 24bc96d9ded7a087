/*
 * mgpu.h -- C ABI of the GB300 path-tracer hot path (libmgpu.so).
 *
 * This is the drop-in boundary beneath Milton's renderer plugin: plain pointers, sizes and
 * status codes, no C++ or torch types.  Every call returns MGPU_OK (0) or a negative
 * MGPU_E_* code; mgpu_last_error() returns a thread-local message for the last failure, the
 * way Milton's SharedLibraryManager::getLastError reports plugin failures
 * (mlt/src/milton/dynamic/SharedLibraryManager.cpp:66-68).
 *
 * Streams are passed as `void*` holding a cudaStream_t (NULL = legacy default stream).
 * Calls on one scene are stream-ordered and not re-entrant across host threads; a scene
 * belongs to the device that was current when it was created.
 *
 * Scene geometry is a world-space triangle soup: Milton's ShapeSet flattened through every
 * shape's transform (mlt/src/milton/shapes/ShapeSet.cpp:36-80, Mesh.cpp:211-251,
 * Transformable.inl:18-48).  The global primitive id of a triangle is its index in that soup:
 * the prefix offset of its shape in ShapeSet order plus its index inside the shape, the pair
 * (pt.shape, pt.index) that kdTreeAccel::getIntersection reports (kdTreeAccel.cpp:991-993).
 */
#ifndef MGPU_H_
#define MGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGPU_OK 0
#define MGPU_E_INVALID (-1)  /* bad argument */
#define MGPU_E_CUDA (-2)     /* CUDA runtime error */
#define MGPU_E_NOMEM (-3)    /* allocation failed (host or device) */
#define MGPU_E_BUDGET (-4)   /* request exceeds the memory budget it was admitted under */
#define MGPU_E_STATE (-5)    /* call not valid in the object's current state */
#define MGPU_E_DEVICE (-6)   /* reserved: kernels stay in bounds by construction (tree depth <= 64
                                checked at build, queue sizes bounded by the wave) and never
                                report a guarded fault today */

/* triangle flags */
#define MGPU_TRI_CULLED 1u   /* back-face culled, Milton `Triangle` (Triangle.cpp:245-272); else two-sided `MeshTriangle` */

/* material types (Material::getBSDF, Material.cpp:67-92) */
#define MGPU_MAT_DIFFUSE 0
#define MGPU_MAT_PHONG 1
#define MGPU_MAT_DIELECTRIC 2

typedef struct mgpu_accel mgpu_accel; /* host-side SAH kd-tree, flattened */
typedef struct mgpu_scene mgpu_scene; /* device-resident scene: tree, triangles, materials, lights */

/* kd-tree build parameters, Milton's SAH (kdTreeAccel.cpp:722-877) with its knobs; Milton's
 * defaults (kdTreeAccel.h:97-104) are min_prims 3, max_depth 24, cost_traversal 1, empty_bias 0.9.
 * threads 0 = all cores.  The renderer's default traversal cost is MGPU_KD_COST_TRAVERSAL (a scene
 * file's kdCostTraversal still sets it): SAH weighs a node step against a triangle test, and on
 * this GPU the traversal kernels test a leaf's triangles with all lanes of a warp but descend
 * nodes with the few lanes whose rays are still descending, so a node step costs about three
 * tests (mid frame: cost 1 / 2 / 3 / 4 / 6 -> 270 / 283 / 288 / 286 / 277 Mpaths/s).  The tree
 * never changes a closest hit (only which of two equal-t triangles is reported).              */
#define MGPU_KD_COST_TRAVERSAL 3.0
typedef struct {
  uint32_t min_prims;
  uint32_t max_depth;
  double cost_traversal;
  double empty_bias;
  uint32_t threads;
} mgpu_kd_params;

/* Milton's kd build log (kdTreeAccel.cpp:460-471), sums instead of averages */
typedef struct {
  uint64_t no_internal, no_leaves, min_depth, max_depth, sum_depth, min_prims, max_prims, sum_prims;
  uint64_t node_pairs, refs, bytes_nodes, bytes_refs;
  double build_seconds;
} mgpu_kd_stats;

/* Scene description, all host pointers.
 *   tri_v      ntri*9 floats, world-space vertices (v0,v1,v2)
 *   tri_n      ntri*9 floats, per-vertex shading normals (unit); NULL = face normals
 *   tri_mat    ntri material indices
 *   tri_light  ntri light indices (-1 = not an emitter); NULL = none
 *   tri_flags  ntri MGPU_TRI_* flags; NULL = all two-sided
 *   materials  nmat*16 floats: type, kd[3], ks[3], n, ior, transparency, then texture slots
 *              [10] kd, [11] ks, [12] transparency, [13] bump map: 1 + index into textures
 *              (0 = none; a textured key replaces the constant, Material::getSpectralSampleSet,
 *              Material.cpp:229-283), [14..15] 0
 *   lights     nlight*16 floats: center[3], ex[3], ez[3], normal[3], area, Le[3]
 *              (a Milton `Plane` under a transform: getPosition(u,v) = center + (u-.5)ex + (v-.5)ez,
 *               Plane.cpp:91-93; Le = power / (area * pi), Emitter.cpp:34-50)
 *   light_ext  NULL (every light is a plane) or nlight*16 floats: type, then per type
 *              MGPU_LIGHT_PLANE     nothing more
 *              MGPU_LIGHT_TRIANGLE  uv0[2], a[2], b[2], 1/|a x b|: a Milton `Triangle`, with center =
 *                                   v1, ex = v2 - v1, ez = v3 - v1 (world), normal its normal, area
 *                                   its object-space area; the light sample (u, v) lands at
 *                                   v1 + |c x b| ex / |a x b| + |c x a| ez / |a x b|, c = (u, v) - uv0,
 *                                   a = uv1 - uv0, b = uv2 - uv0 (Triangle::getPosition,
 *                                   Triangle.cpp:332-354)
 *              MGPU_LIGHT_MESH      [8] first triangle, [9] triangle count (uint32 bit patterns): a
 *                                   Milton `Mesh` emitter over that run of the soup; area = its
 *                                   world-space area; a sample (u, v) picks triangle floor(u count)
 *                                   and lands at barycentrics (r1, v, r2) / (r1 + v + r2) with two
 *                                   more uniforms r1, r2, normal = interpolated vertex normals
 *                                   (Mesh::getPosition / getPoint, Mesh.cpp:436-448,
 *                                   MeshTriangle::getPosition, MeshTriangle.cpp:299-333)
 *              MGPU_LIGHT_SPHERE    [1..4] the object-to-world quaternion, [5] the radius: a Milton
 *                                   `Sphere` emitter at center, sampled as Sphere::getPosition does
 *                                   (Sphere.cpp:114-121: x = clamp(tan((1 - u) / 2 pi)), y =
 *                                   clamp(sin((1/2 - v) / pi) / 2), z = sqrt(1 - x^2 - y^2) in object
 *                                   space, a patch off the sphere's surface), normal = the object
 *                                   point's direction, area = pi (its object-space area, :131-134)
 *              MGPU_LIGHT_POINT     nothing more: a Milton `PointShape` at center, area 0, one
 *                                   light sample, no normal (cosine 1) and no triangles
 *                                   (DirectIllumination.cpp:90-130)
 *              [15] 1 = an OmniEmitter: Le in every direction, both sides (OmniEmitter.cpp);
 *                   0 = OrientedEmitter (the normal's side); points are omni either way
 *   tri_uv     NULL (every uv is (0, 0)) or ntri*6 floats: the uv of each vertex; a hit's uv is
 *              their barycentric interpolation (Shape::_getUV of the shape the triangle came from:
 *              Triangle.cpp:23-39, Plane.cpp:52-59, Cube.cpp:84-105 and Mesh.cpp:408-416 are
 *              all affine over a triangle, so per-vertex uvs reproduce them)
 *   textures   ntex records (mgpu_texture), referenced by the material texture slots
 *   background radiance of rays that leave the scene (Scene::getBackgroundRadiance, Scene.cpp:
 *              116-118, added at every depth; not sampled by next-event estimation):
 *              background_tex = 1 + index of a colour map read as Milton's latitude-longitude
 *              EnvironmentMap (EnvironmentMap.cpp:40-96: the map's texel at the uv of -d), or 0
 *              for the constant background_le (an omni background: power / 4 pi; zeros = the
 *              default black background)
 *   spheres    nsphere (at most MGPU_MAX_SPHERES) analytic Milton `Sphere`s beside the triangle
 *              soup, 8 floats each: center[3], radius, then the unit quaternion (x, y, z, w) that
 *              rotates world directions into the sphere's object frame (for its uvs); primitive
 *              id ntri + index, material sphere_mat[index], light sphere_light[index].  Every ray tests
 *              every sphere (Sphere::getIntersection, Sphere.cpp:17-48), so a scene of many
 *              spheres is better tessellated.                                               */
typedef struct mgpu_texture mgpu_texture;
typedef struct {
  int64_t ntri;
  const float *tri_v;
  const float *tri_n;
  const int32_t *tri_mat;
  const int32_t *tri_light;
  const uint32_t *tri_flags;
  int32_t nmat;
  const float *materials;
  int32_t nlight;
  const float *lights;
  const float *light_ext;
  const float *tri_uv;
  int32_t ntex;
  const mgpu_texture *textures;
  int32_t background_tex;
  float background_le[3];
  int32_t nsphere;
  const float *spheres;
  const int32_t *sphere_mat;
  const int32_t *sphere_light;  /* NULL or nsphere light indices (-1 = not an emitter) */
} mgpu_scene_desc;

/* A material's image map (Material::getSample, Material.cpp:285-301, and the bump map of
 * Material::_initShadingNormal, :179-225).  rgb: width*height*3 linear values, row 0 = the
 * image's first (top) row; 8-bit images are byte / 255 (Rgba32 -> RgbaHDR, Rgba.inl:32-40).
 * A lookup at uv takes texel (floor(clamp(frac(u repeat_u) width, 0, width - 1)), same for v
 * and rows).
 *   MGPU_TEX_COLOR  the texel value is KernelFilter::apply (KernelFilter.cpp:106-140) of the
 *                   image at that texel: sum w(i, j) rgb[clamped row + i, col + j] / sum w with
 *                   the material's filter (type, support, p1, p2 as mgpu_film_set_filter; w =
 *                   filter(i - 1/2, j - 1/2) over the (ceil(support) | 1)^2 offsets, the
 *                   kernel KernelFilter::_computeKernel builds).  Computed once per texel on the
 *                   device when the scene is created.
 *   MGPU_TEX_BUMP   the shading normal becomes normalize(N + bump_intensity (gx U + gy V)), with
 *                   U, V = N's orthonormal basis and gx, gy central luminance differences
 *                   (0.2126 r + 0.7152 g + 0.0722 b) at the texel, clamped at the edges; N
 *                   unchanged where both are 0.  A bump-mapped material may not emit.       */
struct mgpu_texture {
  int32_t width, height;
  const float *rgb;
  int32_t kind;        /* MGPU_TEX_COLOR or MGPU_TEX_BUMP */
  int32_t filter;      /* MGPU_FILTER_BOX .. MGPU_FILTER_LANCZOS_SINC (colour maps) */
  float support, p1, p2;
  float repeat_u, repeat_v;
  float bump_intensity;
};

#define MGPU_TEX_COLOR 0
#define MGPU_TEX_BUMP 1

#define MGPU_MAX_SPHERES 256

#define MGPU_LIGHT_PLANE 0
#define MGPU_LIGHT_TRIANGLE 1
#define MGPU_LIGHT_MESH 2
#define MGPU_LIGHT_POINT 3
#define MGPU_LIGHT_SPHERE 4

/* Render parameters.  Defaults mirror Milton's PathTracer/DirectIllumination keys:
 * noDirectSamples 1, efficientDirect 1, no maximum depth, Russian roulette from depth 2
 * (PathTracer.cpp:88-89).  max_depth > 0 caps the number of path vertices.
 * camera: eye[3], look[3] (unit), up[3], heightAngle (degrees), aspectRatio, then the thin lens:
 * aperture (metres; 0 = pinhole), focal length, focal distance, and two unused floats
 * (ThinLensCamera, ThinLensCamera.cpp:62-175).
 * Sample passes [sample_begin, sample_begin + sample_count) of spp are rendered and added to
 * the film (progressive refinement = further calls with later passes).                    */
typedef struct {
  int32_t width, height;
  int32_t spp;            /* noSuperSamples: sets the stratification side floor(sqrt(spp)) */
  int32_t sample_begin;
  int32_t sample_count;
  int32_t no_direct_samples;
  int32_t max_depth;      /* 0 = unlimited (hard cap 1024, counted) */
  int32_t rr_start_depth; /* Russian roulette applies at depth >= this */
  int32_t efficient_direct;
  int32_t wave_paths;     /* paths in flight per wave; 0 = automatic */
  uint64_t seed;
  uint32_t stream_id;     /* decorrelates independent replicas / jobs */
  float camera[16];
} mgpu_render_params;

typedef struct {
  uint64_t paths, extension_rays, shadow_rays, truncated_paths, bounces, kernel_launches;
} mgpu_render_stats;

/* ---------------------------------------------------------------------------------------- */
const char *mgpu_last_error(void);
int mgpu_version(void);

/* Host SAH kd-tree build over the scene's triangles; replaces kdTreeAccel::init
 * (kdTreeAccel.cpp:403-472) for the flattened soup.  Deterministic for any thread count. */
int mgpu_accel_build(const mgpu_scene_desc *desc, const mgpu_kd_params *params, mgpu_accel **out);
int mgpu_accel_stats(const mgpu_accel *accel, mgpu_kd_stats *out);
/* Depth-first (left before right) serialisation for node-by-node comparison:
 * kind 0..2 = split axis, 3 = leaf; split = stored float split; count = leaf prim count;
 * prims = leaf prim lists in Milton's stored order.  Pass NULL arrays to query sizes.    */
int mgpu_accel_serialize(const mgpu_accel *accel, int32_t *kind, float *split, int32_t *count, int32_t *prims,
                         int64_t *n_nodes, int64_t *n_prims);
int mgpu_accel_destroy(mgpu_accel *accel);

/* Upload accel + scene to the current device.  The triangle arrays uploaded are the ones the
 * accel captured at build time (tree layout with leaf-ordered triangle records, triangles by id,
 * shading records; page-locked on the first upload); desc supplies the materials and lights and
 * must describe the same triangles.  Returns after the copies complete.                   */
int mgpu_scene_create(const mgpu_scene_desc *desc, const mgpu_accel *accel, void *stream, mgpu_scene **out);
int mgpu_scene_destroy(mgpu_scene *scene);
int mgpu_scene_bytes(const mgpu_scene *scene, uint64_t *out);
/* Device bytes mgpu_scene_create would allocate for this accel with nmat materials and nlight
 * lights (admission against a memory budget before uploading).  No reference counterpart. */
int mgpu_accel_device_bytes(const mgpu_accel *accel, int32_t nmat, int32_t nlight, uint64_t *out);
/* The same for a full description, textures and uvs included. */
int mgpu_scene_device_bytes(const mgpu_scene_desc *desc, const mgpu_accel *accel, uint64_t *out);
/* Texel values of texture tex as the device holds them (after filtering): width*height*4
 * floats (colour maps: rgb, 0; bump maps: gx, gy, 0, 0).  Synchronises.  For tests. */
int mgpu_scene_read_texels(const mgpu_scene *scene, int32_t tex, float *out, void *stream);
/* Tuning: how many of the breadth-first top 16-byte pairs the traversal kernels stage in
 * shared memory per block (0 = none; clamped to what the builder laid out breadth-first). */
int mgpu_scene_set_top_pairs(mgpu_scene *scene, uint32_t n);

/* Ray queries on device buffers (Scene::getIntersection / Scene::intersects).
 *   rays: n * 8 floats  (origin xyz, tmin, direction xyz, tmax)
 *   hits: n * 4 floats  (t, prim id as int bits, b1, b2); t = +inf and prim = -1 on a miss
 *   occluded: n bytes   (1 if any hit with tmin < t < tmax)                               */
int mgpu_trace_closest(const mgpu_scene *scene, const float *d_rays, float *d_hits, int64_t n, void *stream);
int mgpu_trace_any(const mgpu_scene *scene, const float *d_rays, uint8_t *d_occluded, int64_t n, void *stream);
/* Same queries with per-ray traversal counters written to d_counts (n * 4 uint32:
 * nodes visited, leaf refs read, triangles tested, max stack depth) -- measurement only. */
int mgpu_trace_closest_counted(const mgpu_scene *scene, const float *d_rays, float *d_hits, uint32_t *d_counts,
                               int64_t n, void *stream);

/* Film: compensated FP32 sums per pixel: (rgb sum, sample count) and (rgb Kahan compensation,
 * sum of squared per-sample luminance (r+g+b)/3, for variance and error estimates).         */
typedef struct mgpu_film mgpu_film;
int mgpu_film_create(int32_t width, int32_t height, void *stream, mgpu_film **out);
int mgpu_film_clear(mgpu_film *film, void *stream);
int mgpu_film_destroy(mgpu_film *film);
/* The film's output in FP64: out = host array of width*height*3 doubles (synchronises): the
 * per-pixel mean, or with a reconstruction filter set, sum(w L) / sum(w) over the samples
 * splatted onto each pixel.  The mean is taken on the device in a scratch buffer of 24 bytes
 * per pixel that the calling thread keeps for its later reads (grown to the largest film it
 * has read, released when the thread exits).                                                */
int mgpu_film_read(mgpu_film *film, double *out_mean, void *stream);
/* Reconstruction filter of ReconstructionRenderOutput (ReconstructionRenderOutput.cpp:30-83):
 * every sample is splatted onto the pixels within (ceil(support) | 1) / 2 of its own with
 * weight filter(pixel - position) when > 0 (the per-pixel mean is kept as well).  type:
 * MGPU_FILTER_NONE, _BOX, _TRIANGLE, _GAUSSIAN (p1 = sigma), _MITCHELL (p1 = B, p2 = C),
 * _LANCZOS_SINC (p1 = tau) (M/filters/KernelFilter.cpp:18-40).  The splat sums are 2^-24
 * fixed point, so results do not depend on the order of the atomic additions.  Clears them. */
int mgpu_film_set_filter(mgpu_film *film, int32_t type, float support, float p1, float p2, void *stream);
#define MGPU_FILTER_NONE 0
#define MGPU_FILTER_BOX 1
#define MGPU_FILTER_TRIANGLE 2
#define MGPU_FILTER_GAUSSIAN 3
#define MGPU_FILTER_MITCHELL 4
#define MGPU_FILTER_LANCZOS_SINC 5
/* Raw device film: 2 float4 per pixel (sum.rgb + count, compensation.rgb + luminance sum of
 * squares) -> host floats.                                                                  */
int mgpu_film_read_raw(mgpu_film *film, float *out8, void *stream);
/* Error estimate of n films in one pass on the device (synchronises): out_rmse[i] =
 * sqrt(mean over pixels with >= 2 samples of var_pixel / n_pixel), var_pixel the sample
 * variance of the per-sample luminance (r+g+b)/3 -- the expected RMSE of the film's mean
 * luminance against the converged image; +inf if no pixel has 2 samples.  Deterministic.
 * Progressive refinement's stopping test; no counterpart in the reference.                */
int mgpu_film_error(mgpu_film *const *films, int32_t n, double *out_rmse, void *stream);
/* Reinhard tone map of the film's output (as mgpu_film_read) to 8-bit sRGB (width*height*4 bytes, RGBA,
 * row-major from the top), computed on the device in FP64 (ReinhardToneMap::map,
 * M/renderers/tonemaps/ReinhardToneMap.cpp:25-94; synchronises).                            */
int mgpu_film_tonemap(mgpu_film *film, uint8_t *out_rgba, void *stream);

/* PathTracer::render over the requested sample passes (PathTracer.cpp:28-116 per path). */
int mgpu_render(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, void *stream);
/* Allocation-free render.  No counterpart in the reference: Milton's renderers allocate freely.
 * Some hosts cannot let a library allocate device memory while they render -- a render
 * server that admits jobs against a fixed HBM budget and forbids allocation after start-up, or
 * a plugin host whose device allocator is its own -- so this entry point renders with the same
 * estimator, random numbers and film as mgpu_render but never calls cudaMalloc, cudaFree or any
 * allocating routine.  Its scratch (path state, ray queues, light-sample slots) is one fixed
 * 32 MiB device array compiled into libmgpu.so; every GPU that loads the library's rendering
 * module holds it until the process exits.  The caller still provides the inputs and outputs: a
 * scene from mgpu_scene_create and a film from mgpu_film_create, made beforehand.
 *   - The scratch bounds the wave: with 4 light samples per vertex it holds about 65 000
 *     paths in flight (wave_paths 0 picks the most that fit), so large frames render slower
 *     than with mgpu_render.  A wave_paths above that capacity is rejected with
 *     MGPU_E_INVALID and a message naming the capacity; nothing is rendered.
 *   - The array comes into existence when the rendering module is loaded on a device.  Under
 *     CUDA's lazy module loading (the default) that is the first render call of any kind on
 *     that device, so the first mgpu_render_noalloc call there may itself take the 32 MiB: a
 *     host that fixes its device-memory budget makes one render call per device at start-up,
 *     before fixing it.  That first call also looks up the array's device address with
 *     cudaGetSymbolAddress; make it before any stream capture.
 *   - The looked-up address stays valid for the life of the process's context on the device:
 *     after cudaDeviceReset every object of this library on that device is invalid, and this
 *     entry point must not be called there again.
 *   - All calls share the one array and it keeps the last call's contents; each call clears
 *     what must start at zero itself.  Calls whose work overlaps on the GPU (other streams,
 *     other host threads) race on the array: serialise them.
 *   - mgpu_render_stats_get and mgpu_render_wave_queues read their numbers from the array
 *     after a call of this entry point, so they report the most recent mgpu_render_noalloc
 *     call on that device, whichever host thread made it.                                  */
int mgpu_render_noalloc(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, void *stream);
/* Batched rendering: render requests of different scenes, resolutions and sample counts share
 * waves, so scenes too small to fill the GPU alone render together; each request's film gets
 * exactly the image mgpu_render would give it.  With every request at a fixed max_depth the
 * whole launch sequence is captured in one CUDA graph and launched once (use_graph = 1).
 * No counterpart in the reference (Milton renders one scene per process).                  */
typedef struct mgpu_batch mgpu_batch;
int mgpu_batch_create(mgpu_batch **out);
int mgpu_batch_add(mgpu_batch *batch, const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film);
int mgpu_batch_set(mgpu_batch *batch, int64_t wave_paths, int32_t use_graph); /* wave_paths 0 = automatic */
int mgpu_batch_render(mgpu_batch *batch, void *stream);
int mgpu_batch_clear(mgpu_batch *batch);
int mgpu_batch_destroy(mgpu_batch *batch);
/* Render and also write every path's radiance (after Milton's specular channel masking)
 * to d_path_L: (pixel * sample_count + sample) * 4 floats.  Test/measurement helper.     */
int mgpu_render_paths(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, float *d_path_L,
                      void *stream);
int mgpu_render_stats_get(mgpu_render_stats *out); /* stats of the last render on this thread (synchronises) */
/* Queue sizes per bounce of the last wave of the last render on this thread (synchronises):
 * ext[b] = live paths traced at bounce b, shadow[b] = shadow rays queued at bounce b.       */
int mgpu_render_wave_queues(uint32_t *ext, uint32_t *shadow, int32_t max_bounces);
/* Render with traversal counters: counts8 = extension {nodes, leaf refs, triangles, rays},
 * shadow {nodes, leaf refs, triangles, rays} summed over the render (synchronises).
 * Measurement helper for the memory roofline; slower than mgpu_render.                   */
int mgpu_render_counted(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, uint64_t *counts8,
                        void *stream);
/* Per-kernel timing: when enabled, every render launch on this thread is bracketed by CUDA
 * events on its stream.  mgpu_profile_read (synchronises) returns milliseconds and launch
 * counts per kernel class: generate, extend, shade, shadow, accumulate, queue binning.
 * Enabling resets. */
int mgpu_profile_enable(int enable);
int mgpu_profile_read(double *ms6, uint64_t *launches6);
/* Process-wide tuning knobs (results do not depend on them):
 *   "persistent"     0/1  persistent warp-level traversal with per-lane ray refill (default 0)
 *   "coop_leaf"      0..3 warp-shared leaf tests: the triangles of all the lanes' current leaves
 *                    are tested by the whole warp, 32 at a time; bit 0 = shadow (any-hit)
 *                    kernel, bit 1 = extension (closest-hit) kernel (default 3: both)
 *   "trav_block"     64 / 128 / 256  threads per block of the grid-stride and warp-shared
 *                    traversal kernels, at the same threads (and registers) per SM (default 256)
 *   "bin_shadow"     0/1  counting-sort shadow rays by (light, origin cell) (default 1)
 *   "bin_extension"  0/1  counting-sort extension rays by (direction octant, origin cell) (default 1)
 *   "bin_min_paths"  n    waves of fewer paths are not binned (default 2^22)
 *   "carveout"       -2..100  shared-memory carveout (percent) preferred for the traversal and
 *                    shade kernels: -2 = per kernel, the least shared memory that keeps all its
 *                    register-limited resident blocks, the rest of the SM's memory as L1
 *                    (default); -1 = the driver's choice; applied on each device before its next
 *                    render                                                                     */
int mgpu_tune_set(const char *key, int64_t value);
int mgpu_tune_get(const char *key, int64_t *value);

/* Read bandwidth of this device (measurement only, no counterpart in the reference): one
 * launch reads a `bytes` buffer (cudaMalloc'd here; >= 4096, a multiple of 16) `reps` times
 * through L2-only loads; *gbs = bytes * reps / time.  A buffer that fits the L2 measures the L2's
 * read bandwidth (the denominator of the traversal kernels' L2 roofline), a larger one the HBM's.
 * Synchronises. */
int mgpu_measure_read_bandwidth(uint64_t bytes, int32_t reps, double *gbs, void *stream);

/* Kernel launches issued by this library since load (for launch accounting). */
uint64_t mgpu_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* MGPU_H_ */
