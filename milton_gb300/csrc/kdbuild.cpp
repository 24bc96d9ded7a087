// kdbuild.cpp -- host SAH kd-tree build with Milton's split semantics, parallel over subtrees,
// flattened into 16-byte sibling-pair records for the GPU traversal.
//
// Split selection follows kdTreeAccel::_computeSplitPlaneSAH (kdTreeAccel.cpp:722-811): every
// axis except the parent's split axis, candidate planes at primitive AABB extrema with
// min/max/planar events, cost SA_L*(n_L+n_P) + SA_R*n_R scaled by kdEmptyBias when a side is
// empty (:855-877), leaf when the best cost exceeds (n - kdCostTraversal)*SA (:793-804).
// Partition and termination follow _buildTree (:533-630).  Because every candidate position is
// a float vertex coordinate, positions are sorted as 62-bit integer keys instead of
// (double, enum) pairs; the grouping of equal positions, and therefore every cost, split and
// leaf, is the same as the reference's std::sort sweep.  Subtrees are built on separate threads;
// the result does not depend on the thread count.
#include "kdbuild.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <memory>
#include <thread>

namespace mgpu {

void KdLog::merge(const KdLog &o) {
  no_internal += o.no_internal;
  no_leaves += o.no_leaves;
  min_depth = std::min(min_depth, o.min_depth);
  max_depth = std::max(max_depth, o.max_depth);
  sum_depth += o.sum_depth;
  min_prims = std::min(min_prims, o.min_prims);
  max_prims = std::max(max_prims, o.max_prims);
  sum_prims += o.sum_prims;
}

namespace {

struct Box {
  double mn[3], mx[3];
};

struct Node {
  bool leaf = true;
  int axis = 0;
  float split = 0.0f;
  std::unique_ptr<Node[]> kids;
  std::vector<int32_t> prims;
};

inline uint32_t order_bits(float f) {
  if (f == 0.0f) f = 0.0f;  // -0 and +0 are one plane position
  uint32_t u;
  memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

inline double box_area(const Box &b) {
  double d0 = b.mx[0] - b.mn[0], d1 = b.mx[1] - b.mn[1], d2 = b.mx[2] - b.mn[2];
  return 2 * (d0 * d1 + d1 * d2 + d2 * d0);
}

inline void split_areas(const Box &b, int axis, double pos, double &l, double &r) {
  double d[3] = {b.mx[0] - b.mn[0], b.mx[1] - b.mn[1], b.mx[2] - b.mn[2]};
  d[axis] = pos - b.mn[axis];
  l = 2 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
  d[axis] = b.mx[axis] - pos;
  r = 2 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
}

struct Shared {
  const float *tmin;  // ntri*3 triangle AABB minima (float)
  const float *tmax;
  const uint8_t *point;
  KdParams p;
  std::atomic<int> spare_threads;
};

constexpr size_t kSpawnMin = 4096;       // subtrees smaller than this stay on the calling thread
constexpr size_t kAxisThreadMin = 262144;  // nodes at least this large evaluate their axes in parallel
constexpr size_t kRadixMin = 65536;        // event lists at least this long are radix sorted

// LSD radix sort of 64-bit keys, 11-bit digits; digits that are equal in every key are skipped.
// Produces the same order as std::sort (a total order on the integers).
void radix_sort(std::vector<uint64_t> &a, std::vector<uint64_t> &tmp) {
  constexpr int kBits = 11, kDigits = (64 + kBits - 1) / kBits;
  constexpr uint32_t kMask = (1u << kBits) - 1u;
  const size_t n = a.size();
  std::vector<uint32_t> hist((size_t)kDigits << kBits, 0u);
  for (size_t i = 0; i < n; ++i) {
    const uint64_t k = a[i];
    for (int d = 0; d < kDigits; ++d) ++hist[((size_t)d << kBits) + ((k >> (d * kBits)) & kMask)];
  }
  tmp.resize(n);
  uint64_t *src = a.data(), *dst = tmp.data();
  for (int d = 0; d < kDigits; ++d) {
    uint32_t *h = &hist[(size_t)d << kBits];
    if (h[(src[0] >> (d * kBits)) & kMask] == n) continue;  // one bucket holds every key
    uint32_t sum = 0;
    for (uint32_t b = 0; b <= kMask; ++b) {
      const uint32_t c = h[b];
      h[b] = sum;
      sum += c;
    }
    for (size_t i = 0; i < n; ++i) dst[h[(src[i] >> (d * kBits)) & kMask]++] = src[i];
    std::swap(src, dst);
  }
  if (src != a.data()) a.swap(tmp);
}

class Task {
 public:
  explicit Task(Shared *s) : s_(s) {}
  KdLog log;

  void leaf(Node *nd, std::vector<int32_t> &&prims, unsigned depth) {
    nd->leaf = true;
    nd->prims = std::move(prims);
    uint64_t n = nd->prims.size();
    log.no_leaves++;
    log.min_prims = std::min<uint64_t>(log.min_prims, n);
    log.max_prims = std::max<uint64_t>(log.max_prims, n);
    log.sum_prims += n;
    log.min_depth = std::min<uint64_t>(log.min_depth, depth);
    log.max_depth = std::max<uint64_t>(log.max_depth, depth);
    log.sum_depth += depth;
  }

  void helper(Node *nd, std::vector<int32_t> &&prims, int parent_axis, unsigned depth, Box box) {
    if (!prims.empty()) build(nd, std::move(prims), parent_axis, depth, box);
    else leaf(nd, std::move(prims), depth);
  }

  void build(Node *nd, std::vector<int32_t> &&prims, int parent_axis, unsigned depth, Box box) {
    const KdParams &p = s_->p;
    const size_t n = prims.size();
    if (depth > log.max_depth) log.max_depth = depth;
    if (n < p.min_prims || depth >= p.max_depth) {
      leaf(nd, std::move(prims), depth);
      return;
    }
    // each axis' best plane (axes in parallel for large nodes), then the first axis whose cost
    // is strictly lowest, as the reference's sequential loop picks it
    double cost_ax[3] = {INFINITY, INFINITY, INFINITY}, pos_ax[3] = {0, 0, 0};
    int axes[3], na = 0;
    for (int axis = 0; axis < 3; ++axis)
      if (axis != parent_axis && box.mn[axis] < box.mx[axis]) axes[na++] = axis;
    if (n >= kAxisThreadMin && na > 1) {
      std::thread th[2];
      bool spawned[2] = {false, false};
      std::vector<uint64_t> keys_extra[2], tmp_extra[2];
      for (int k = 1; k < na; ++k) {
        if (!take_thread()) continue;
        spawned[k - 1] = true;
        const int axis = axes[k];
        th[k - 1] = std::thread([&, axis, k]() {
          best_plane(prims, axis, box, keys_extra[k - 1], tmp_extra[k - 1], cost_ax[axis], pos_ax[axis]);
        });
      }
      best_plane(prims, axes[0], box, keys_, tmp_, cost_ax[axes[0]], pos_ax[axes[0]]);
      for (int k = 1; k < na; ++k) {
        if (spawned[k - 1]) {
          th[k - 1].join();
          s_->spare_threads.fetch_add(1);
        } else {
          best_plane(prims, axes[k], box, keys_, tmp_, cost_ax[axes[k]], pos_ax[axes[k]]);
        }
      }
    } else {
      for (int k = 0; k < na; ++k) best_plane(prims, axes[k], box, keys_, tmp_, cost_ax[axes[k]], pos_ax[axes[k]]);
    }
    double best_cost = INFINITY, best_pos = 0;
    int best_axis = 0;
    for (int axis = 0; axis < 3; ++axis)
      if (cost_ax[axis] < best_cost) { best_cost = cost_ax[axis]; best_pos = pos_ax[axis]; best_axis = axis; }
    if (best_cost == INFINITY) { leaf(nd, std::move(prims), depth); return; }
    double leaf_cost = ((double)(int)n - p.cost_traversal) * box_area(box);
    if (best_cost > leaf_cost) { leaf(nd, std::move(prims), depth); return; }

    std::vector<int32_t> lp, rp;
    lp.reserve(n);
    rp.reserve(n);
    for (size_t i = 0; i < n; ++i) {
      int32_t t = prims[i];
      if (s_->point[t]) continue;
      double mn = s_->tmin[3 * (size_t)t + best_axis], mx = s_->tmax[3 * (size_t)t + best_axis];
      if (mx > best_pos) rp.push_back(t);
      if (mn <= best_pos) lp.push_back(t);
    }
    if (lp.size() == n && rp.size() == n) { leaf(nd, std::move(prims), depth); return; }
    std::vector<int32_t>().swap(prims);
    nd->leaf = false;
    nd->axis = best_axis;
    nd->split = (float)best_pos;
    nd->kids.reset(new Node[2]);
    log.no_internal++;
    Box lb = box, rb = box;
    lb.mx[best_axis] = best_pos;
    rb.mn[best_axis] = best_pos;
    Node *kids = nd->kids.get();
    // left subtree on a new thread when it is large and a thread is spare
    if (lp.size() >= kSpawnMin && rp.size() >= kSpawnMin && take_thread()) {
      std::unique_ptr<Task> sub(new Task(s_));
      std::vector<int32_t> lmove = std::move(lp);
      std::thread th([&sub, kids, &lmove, best_axis, depth, lb]() {
        sub->helper(&kids[0], std::move(lmove), best_axis, depth + 1, lb);
      });
      helper(&kids[1], std::move(rp), best_axis, depth + 1, rb);
      th.join();
      s_->spare_threads.fetch_add(1);
      log.merge(sub->log);
    } else {
      helper(&kids[0], std::move(lp), best_axis, depth + 1, lb);
      helper(&kids[1], std::move(rp), best_axis, depth + 1, rb);
    }
  }

 private:
  // _computeSplitPlaneSAH for one axis (kdTreeAccel.cpp:722-811): sorted min / planar / max
  // events, sweep with SAH cost SA_L (n_L + n_P) + SA_R n_R, empty-side bias
  void best_plane(const std::vector<int32_t> &prims, int axis, const Box &box, std::vector<uint64_t> &keys,
                  std::vector<uint64_t> &tmp, double &best_cost, double &best_pos) const {
    const KdParams &p = s_->p;
    const size_t n = prims.size();
    keys.clear();
    for (size_t i = n; i--;) {
      int32_t t = prims[i];
      if (s_->point[t]) continue;
      float mn = s_->tmin[3 * (size_t)t + axis], mx = s_->tmax[3 * (size_t)t + axis];
      if (mn == mx) {
        keys.push_back(((uint64_t)order_bits(mn) << 2) | 1u);
      } else {
        keys.push_back(((uint64_t)order_bits(mn) << 2) | 2u);
        keys.push_back(((uint64_t)order_bits(mx) << 2) | 0u);
      }
    }
    const size_t m = keys.size();
    if (m == 0) return;
    if (m >= kRadixMin) radix_sort(keys, tmp);
    else std::sort(keys.begin(), keys.end());
    size_t idx = 0;
    uint64_t nl = 0, nr = n;
    while (idx < m - 1) {
      uint64_t cur = keys[idx] >> 2;
      uint64_t cnt[3] = {0, 0, 0};
      do {
        ++cnt[keys[idx] & 3u];
      } while (idx < m - 1 && (keys[++idx] >> 2) == cur);
      uint64_t np = cnt[1];
      nr -= cnt[0] + np;
      uint32_t ob = (uint32_t)cur;
      uint32_t fb = (ob & 0x80000000u) ? (ob & 0x7FFFFFFFu) : ~ob;
      float fpos;
      memcpy(&fpos, &fb, 4);
      double pos = fpos;
      if (pos > box.mn[axis] && pos < box.mx[axis]) {
        double la, ra;
        split_areas(box, axis, pos, la, ra);
        unsigned l = (unsigned)(nl + np);
        double cost = la * l + ra * (unsigned)nr;
        if (l + np == 0 || nr == 0) cost *= p.empty_bias;
        if (cost < best_cost) { best_cost = cost; best_pos = pos; }
      }
      nl += cnt[2] + np;
    }
  }

  bool take_thread() {
    int cur = s_->spare_threads.load();
    while (cur > 0) {
      if (s_->spare_threads.compare_exchange_weak(cur, cur - 1)) return true;
    }
    return false;
  }
  Shared *s_;
  std::vector<uint64_t> keys_, tmp_;
};

// -------------------------------------------------------------------------------------------
// flattening
struct Flattener {
  KdTree &out;
  explicit Flattener(KdTree &o) : out(o) {}

  // writes the slot for node nd; child pairs are allocated by the caller's traversal order
  void write_leaf(uint32_t slot, const Node *nd) {
    uint32_t count = (uint32_t)nd->prims.size();
    uint32_t w0 = (count << 2) | kLeafTag, w1 = 0;
    if (count == 1) {
      w1 = (uint32_t)nd->prims[0];
    } else if (count > 1) {
      w1 = (uint32_t)out.refs.size();
      for (uint32_t i = count; i--;) out.refs.push_back((uint32_t)nd->prims[i]);
    }
    set(slot, w0, w1);
  }
  void set(uint32_t slot, uint32_t w0, uint32_t w1) {
    Pair &p = out.pairs[slot >> 1];
    if (slot & 1u) { p.b0 = w0; p.b1 = w1; } else { p.a0 = w0; p.a1 = w1; }
  }
  uint32_t alloc_pair() {
    Pair z; z.a0 = kLeafTag; z.a1 = 0; z.b0 = kLeafTag; z.b1 = 0;
    out.pairs.push_back(z);
    return (uint32_t)(out.pairs.size() - 1);
  }
  void interior(uint32_t slot, const Node *nd, uint32_t child_pair) {
    uint32_t sb;
    memcpy(&sb, &nd->split, 4);
    set(slot, (child_pair << 2) | (uint32_t)nd->axis, sb);
  }
  // depth-first layout of a subtree whose root slot is already reserved
  void dfs(uint32_t slot, const Node *nd) {
    if (nd->leaf) { write_leaf(slot, nd); return; }
    uint32_t cp = alloc_pair();
    interior(slot, nd, cp);
    dfs(2 * cp, &nd->kids[0]);
    dfs(2 * cp + 1, &nd->kids[1]);
  }
  void run(const Node *root, uint32_t top_limit) {
    out.pairs.clear();
    out.refs.clear();
    alloc_pair();  // pair 0: root + unused
    std::vector<std::pair<uint32_t, const Node *>> level, next;
    level.push_back({0u, root});
    // breadth-first while the top fits the staging budget
    while (!level.empty()) {
      size_t interior_here = 0;
      for (auto &e : level) interior_here += e.second->leaf ? 0 : 1;
      if (out.pairs.size() + interior_here > top_limit) break;
      next.clear();
      for (auto &e : level) {
        if (e.second->leaf) { write_leaf(e.first, e.second); continue; }
        uint32_t cp = alloc_pair();
        interior(e.first, e.second, cp);
        next.push_back({2 * cp, &e.second->kids[0]});
        next.push_back({2 * cp + 1, &e.second->kids[1]});
      }
      level.swap(next);
    }
    out.top_pairs = (uint32_t)out.pairs.size();
    for (auto &e : level) dfs(e.first, e.second);
  }
};

void ser(const KdTree &t, uint32_t w0, uint32_t w1, int32_t *kind, float *split, int32_t *count, int32_t *prims,
         int64_t &ni, int64_t &np) {
  int64_t i = ni++;
  if ((w0 & 3u) == kLeafTag) {
    uint32_t c = w0 >> 2;
    if (kind) { kind[i] = 3; split[i] = 0.0f; count[i] = (int32_t)c; }
    if (c == 1) {
      if (prims) prims[np] = (int32_t)w1;
      ++np;
    } else {
      // stored reversed: emit in Milton's list order
      for (uint32_t k = 0; k < c; ++k) {
        if (prims) prims[np] = (int32_t)t.refs[w1 + (c - 1 - k)];
        ++np;
      }
    }
    return;
  }
  if (kind) { kind[i] = (int32_t)(w0 & 3u); memcpy(&split[i], &w1, 4); count[i] = 0; }
  const Pair &p = t.pairs[w0 >> 2];
  ser(t, p.a0, p.a1, kind, split, count, prims, ni, np);
  ser(t, p.b0, p.b1, kind, split, count, prims, ni, np);
}

}  // namespace

bool kd_build(const float *v, int64_t ntri, const KdParams &p, KdTree &out, const char **err) {
  auto t_start = std::chrono::steady_clock::now();
  if (ntri < 0 || ntri > (int64_t)0x3FFFFFFF) { *err = "triangle count out of range"; return false; }
  if (p.max_depth > (uint32_t)kMaxStack) { *err = "kdMaxDepth exceeds the traversal stack (64)"; return false; }
  if (p.min_prims < 1) { *err = "kdMinPrimitives must be >= 1"; return false; }
  std::vector<float> tmn((size_t)ntri * 3), tmx((size_t)ntri * 3);
  std::vector<uint8_t> point((size_t)ntri);
  Box root;
  for (int k = 0; k < 3; ++k) { root.mn[k] = INFINITY; root.mx[k] = -INFINITY; }
  for (int64_t t = 0; t < ntri; ++t) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        float x = v[t * 9 + j * 3 + k];
        if (!(x == x) || fabsf(x) > 3.0e37f) { *err = "non-finite vertex coordinate"; return false; }
        mn[k] = std::min(mn[k], x);
        mx[k] = std::max(mx[k], x);
      }
    bool is_point = mn[0] == mx[0] && mn[1] == mx[1] && mn[2] == mx[2];
    point[t] = is_point ? 1 : 0;
    for (int k = 0; k < 3; ++k) { tmn[3 * t + k] = mn[k]; tmx[3 * t + k] = mx[k]; }
    // SpatialAccel::init adds non-point boxes; AABB::add(AABB) skips boxes whose min and max
    // compare equal under Milton's fuzzy EQ (AABB.inl:67-72, utilities.h:240)
    if (!is_point) {
      bool same = true;
      for (int k = 0; k < 3; ++k) {
        double a = mn[k], b = mx[k];
        bool eq = fabs(a - b) < 1e-7 || (fabs(a - b / ((fabs(b) > fabs(a)) ? b : a)) <= 1e-7);
        same = same && eq;
      }
      if (!same)
        for (int k = 0; k < 3; ++k) {
          root.mn[k] = std::min(root.mn[k], (double)mn[k]);
          root.mx[k] = std::max(root.mx[k], (double)mx[k]);
        }
    }
  }
  Shared sh;
  sh.tmin = tmn.data();
  sh.tmax = tmx.data();
  sh.point = point.data();
  sh.p = p;
  unsigned hw = std::thread::hardware_concurrency();
  unsigned nth = p.threads ? p.threads : (hw ? hw : 1);
  sh.spare_threads.store((int)nth - 1);
  Node rootn;
  Task task(&sh);
  std::vector<int32_t> prims((size_t)ntri);
  for (int64_t i = 0; i < ntri; ++i) prims[i] = (int32_t)i;
  if (ntri > 0) task.build(&rootn, std::move(prims), 3, 0, root);
  else task.leaf(&rootn, std::move(prims), 0);
  out.log = task.log;
  for (int k = 0; k < 3; ++k) {
    out.bmin[k] = ntri > 0 ? root.mn[k] : 0.0;
    out.bmax[k] = ntri > 0 ? root.mx[k] : 0.0;
  }
  Flattener fl(out);
  fl.run(&rootn, std::max<uint32_t>(1u, p.top_pairs));
  if (out.pairs.size() >= (1ull << 30) || out.refs.size() >= (1ull << 32)) {
    *err = "tree too large for the 30-bit pair index";
    return false;
  }
  out.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return true;
}

void kd_device_layout(const KdTree &t, const float *v, const uint32_t *flags, std::vector<Pair> &pairs_out,
                      std::vector<F4> &ltris_out) {
  pairs_out = t.pairs;
  ltris_out.clear();
  size_t nref = 0;
  for (const Pair &p : t.pairs) {
    if ((p.a0 & 3u) == kLeafTag) nref += p.a0 >> 2;
    if ((p.b0 & 3u) == kLeafTag) nref += p.b0 >> 2;
  }
  ltris_out.reserve(nref * 3);
  auto emit = [&](uint32_t &w0, uint32_t &w1) {
    if ((w0 & 3u) != kLeafTag) return;
    uint32_t count = w0 >> 2;
    uint32_t first = (uint32_t)(ltris_out.size() / 3);
    for (uint32_t i = 0; i < count; ++i) {
      uint32_t tri = count == 1 ? w1 : t.refs[(size_t)w1 + i];
      const float *p = v + (size_t)tri * 9;
      uint32_t fl = flags ? flags[tri] : 0u;
      F4 a, b, c;
      a.x = p[0]; a.y = p[1]; a.z = p[2]; memcpy(&a.w, &tri, 4);
      b.x = p[3]; b.y = p[4]; b.z = p[5]; memcpy(&b.w, &fl, 4);
      c.x = p[6]; c.y = p[7]; c.z = p[8]; c.w = 0.0f;
      ltris_out.push_back(a);
      ltris_out.push_back(b);
      ltris_out.push_back(c);
    }
    w1 = count ? first : 0u;
  };
  for (Pair &p : pairs_out) {
    emit(p.a0, p.a1);
    emit(p.b0, p.b1);
  }
}

void kd_serialize(const KdTree &t, int32_t *kind, float *split, int32_t *count, int32_t *prims, int64_t *n_nodes,
                  int64_t *n_prims) {
  int64_t ni = 0, np = 0;
  if (!t.pairs.empty()) ser(t, t.pairs[0].a0, t.pairs[0].a1, kind, split, count, prims, ni, np);
  if (n_nodes) *n_nodes = ni;
  if (n_prims) *n_prims = np;
}

}  // namespace mgpu
