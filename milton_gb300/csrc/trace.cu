// trace.cu -- closest-hit and any-hit ray queries over the flattened kd-tree (sm_103a).
//
// One thread per ray, persistent grid-stride launch sized to the SM count.  Rays are read as
// two 128-bit loads (origin+tmin, direction+tmax) and hits written as one 128-bit store.  The
// breadth-first top of the tree (scene->top_pairs 16-byte pairs) is staged in shared memory
// per block; deeper pairs, leaf lists and triangles go through the read-only data path.
#include "common.cuh"

namespace mgpu {

constexpr int kTraceBlock = 128;

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) k_trace(SceneView s, uint32_t ntop, const float4 *__restrict__ rays,
                                                      float4 *__restrict__ hits, uint8_t *__restrict__ occ,
                                                      uint4 *__restrict__ counts, uint32_t n, uint32_t *fetch) {
  extern __shared__ uint4 smem_top[];
  for (uint32_t i = threadIdx.x; i < ntop; i += blockDim.x)
    smem_top[i] = __ldg(reinterpret_cast<const uint4 *>(s.pairs) + i);
  __syncthreads();
  const Pair *top = ntop ? reinterpret_cast<const Pair *>(smem_top) : nullptr;
  TraceCounts c = {0, 0, 0, 0};
  uint32_t done = 0;
  auto load = [&](uint32_t i, Ray &r) {
    float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
    r.o = v3(a.x, a.y, a.z);
    r.tmin = a.w;
    r.d = v3(b.x, b.y, b.z);
    r.tmax = b.w;
    if (COUNT) c = TraceCounts{0, 0, 0, 0};
  };
  auto store = [&](uint32_t i, bool hit, const TravState &st) {
    if (ANY) {
      occ[i] = hit ? 1 : 0;
    } else {
      hits[i] = make_float4(hit ? st.best : INFINITY, __int_as_float(hit ? st.best_prim : -1), hit ? st.bb1 : 0.0f,
                            hit ? st.bb2 : 0.0f);
    }
    if (COUNT) counts[i] = make_uint4(c.nodes, c.refs, c.tris, c.max_stack);
  };
  auto view = [&](uint32_t) -> const SceneView & { return s; };
  persistent_trace<ANY, COUNT, true>(view, top, ntop, n, fetch, load, store, &c, done);
}

template <bool ANY, bool COUNT>
static int launch_trace(const mgpu_scene *s, const float *rays, float *hits, uint8_t *occ, uint32_t *counts, int64_t n,
                        void *stream) {
  if (!s) return fail(MGPU_E_INVALID, "trace: null scene");
  if (n < 0) return fail(MGPU_E_INVALID, "trace: negative ray count");
  if (n == 0) return MGPU_OK;
  if (n > (int64_t)0xFFFFFFFF) return fail(MGPU_E_INVALID, "trace: more than 2^32 - 1 rays in one call");
  if (!rays || (ANY ? !occ : !hits) || (COUNT && !counts)) return fail(MGPU_E_INVALID, "trace: null buffer");
  if (((uintptr_t)rays & 15) || (!ANY && ((uintptr_t)hits & 15)) || (COUNT && ((uintptr_t)counts & 15)))
    return fail(MGPU_E_INVALID, "trace: ray/hit/count buffers must be 16-byte aligned");
  uint32_t ntop = s->top_pairs;
  size_t smem = (size_t)ntop * sizeof(uint4);
  auto kern = k_trace<ANY, COUNT>;
  if (smem > 48 * 1024) MGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  MGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTraceBlock, smem));
  if (per_sm < 1) per_sm = 1;
  int64_t want = (n + kTraceBlock - 1) / kTraceBlock;
  int64_t grid = std::min<int64_t>(want, (int64_t)device_sm_count() * per_sm);
  MGPU_CUDA(cudaMemsetAsync(s->d_err + 1, 0, sizeof(uint32_t), as_stream(stream)));
  kern<<<(unsigned)grid, kTraceBlock, smem, as_stream(stream)>>>(s->view, ntop, (const float4 *)rays, (float4 *)hits,
                                                                  occ, (uint4 *)counts, (uint32_t)n, s->d_err + 1);
  g_launches.fetch_add(1);
  MGPU_CUDA(cudaGetLastError());
  return MGPU_OK;
}

}  // namespace mgpu

using namespace mgpu;

extern "C" {

int mgpu_trace_closest(const mgpu_scene *scene, const float *d_rays, float *d_hits, int64_t n, void *stream) {
  return launch_trace<false, false>(scene, d_rays, d_hits, nullptr, nullptr, n, stream);
}

int mgpu_trace_any(const mgpu_scene *scene, const float *d_rays, uint8_t *d_occluded, int64_t n, void *stream) {
  return launch_trace<true, false>(scene, d_rays, nullptr, d_occluded, nullptr, n, stream);
}

int mgpu_trace_closest_counted(const mgpu_scene *scene, const float *d_rays, float *d_hits, uint32_t *d_counts,
                               int64_t n, void *stream) {
  return launch_trace<false, true>(scene, d_rays, d_hits, nullptr, d_counts, n, stream);
}

}  // extern "C"
