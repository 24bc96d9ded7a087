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
                                                      uint4 *__restrict__ counts, int64_t n) {
  extern __shared__ uint4 smem_top[];
  for (uint32_t i = threadIdx.x; i < ntop; i += blockDim.x)
    smem_top[i] = __ldg(reinterpret_cast<const uint4 *>(s.pairs) + i);
  __syncthreads();
  const Pair *top = reinterpret_cast<const Pair *>(smem_top);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
    Ray r;
    r.o = v3(a.x, a.y, a.z);
    r.tmin = a.w;
    r.d = v3(b.x, b.y, b.z);
    r.tmax = b.w;
    Hit h;
    TraceCounts c = {0, 0, 0, 0};
    bool hit = traverse<ANY, COUNT>(s, r, h, ntop ? top : nullptr, ntop, &c);
    if (ANY) {
      occ[i] = hit ? 1 : 0;
    } else {
      hits[i] = make_float4(hit ? h.t : INFINITY, __int_as_float(hit ? h.prim : -1), h.b1, h.b2);
    }
    if (COUNT) counts[i] = make_uint4(c.nodes, c.refs, c.tris, c.max_stack);
  }
}

template <bool ANY, bool COUNT>
static int launch_trace(const mgpu_scene *s, const float *rays, float *hits, uint8_t *occ, uint32_t *counts, int64_t n,
                        void *stream) {
  if (!s) return fail(MGPU_E_INVALID, "trace: null scene");
  if (n < 0) return fail(MGPU_E_INVALID, "trace: negative ray count");
  if (n == 0) return MGPU_OK;
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
  kern<<<(unsigned)grid, kTraceBlock, smem, as_stream(stream)>>>(s->view, ntop, (const float4 *)rays, (float4 *)hits,
                                                                  occ, (uint4 *)counts, n);
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
