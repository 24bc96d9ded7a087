// kdbuild.h -- host SAH kd-tree builder and flattener (product side).
#pragma once

#include <stdint.h>

#include <vector>

#include "hd_trace.h"

namespace mgpu {

struct KdParams {
  uint32_t min_prims = 3;     // kdMinPrimitives
  uint32_t max_depth = 24;    // kdMaxDepth
  double cost_traversal = 1;  // kdCostTraversal
  double empty_bias = 0.9;    // kdEmptyBias
  uint32_t threads = 0;       // 0 = hardware concurrency
  uint32_t top_pairs = 2048;  // pairs laid out breadth-first (staged in shared memory)
};

struct KdLog {
  uint64_t no_internal = 0, no_leaves = 0, min_depth = ~0ull, max_depth = 0, sum_depth = 0;
  uint64_t min_prims = ~0ull, max_prims = 0, sum_prims = 0;
  void merge(const KdLog &o);
};

struct KdTree {
  std::vector<Pair> pairs;      // pair 0 = {root, unused}
  std::vector<uint32_t> refs;   // reversed leaf lists (count > 1 only)
  double bmin[3], bmax[3];
  uint32_t top_pairs = 0;       // pairs [0, top_pairs) are the breadth-first top of the tree
  KdLog log;
  double build_seconds = 0;
};

// Builds the tree over ntri triangles (v: ntri*9 floats).  Returns false and sets err on
// invalid parameters.
bool kd_build(const float *v, int64_t ntri, const KdParams &p, KdTree &out, const char **err);

// Depth-first (left before right) serialisation of the flattened tree; prims in Milton's
// stored order.  Pass null arrays to count only.
void kd_serialize(const KdTree &t, int32_t *kind, float *split, int32_t *count, int32_t *prims, int64_t *n_nodes,
                  int64_t *n_prims);

// Device layout: a copy of the pair records whose leaf slots point into ltris (w1 = first
// record), and the leaf triangle records themselves (3 x F4 each: (v0, prim id), (v1, flags),
// (v2, 0)), leaves in pair order, each leaf's run in the reversed (Milton iteration) order.
void kd_device_layout(const KdTree &t, const float *v, const uint32_t *flags, std::vector<Pair> &pairs_out,
                      std::vector<F4> &ltris_out);

}  // namespace mgpu
