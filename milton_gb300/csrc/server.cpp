// server.cpp -- continuous-batching render service (include/mgpu_server.h).
//
// Host-side scheduler over the public C ABI: kd-trees are built by a small pool of background
// threads (mgpu_accel_build), scenes are uploaded on admission (mgpu_scene_create) and evicted
// when idle, and every tick renders the sample passes of all active jobs as one batch
// (mgpu_batch_*), followed by one error-estimate pass over the films at a checkpoint
// (mgpu_film_error).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mgpu_server.h"

namespace mgpu {
int fail(int code, const std::string &msg);
}

namespace {

enum SceneState { kIdle = 0, kBuilding = 1, kBuilt = 2, kBuildFailed = 3 };

struct SrvScene {
  int64_t ntri = 0;
  std::vector<float> v, n, mats, lights, light_ext, uv;
  std::vector<int32_t> mat, light;
  std::vector<uint32_t> flags;
  std::vector<std::vector<float>> tex_rgb;  // owned texel data of each texture
  std::vector<mgpu_texture> tex;
  int32_t bg_tex = 0;
  float bg_le[3] = {0, 0, 0};
  std::vector<float> sph;
  std::vector<int32_t> sph_mat, sph_light;
  int32_t nmat = 0, nlight = 0;
  // written by a build thread, read under the server mutex
  int state = kIdle;
  std::string error;
  mgpu_accel *accel = nullptr;
  uint64_t dev_bytes = 0;
  // stepping thread only
  mgpu_scene *dev = nullptr;
  int active = 0;
  uint64_t last_use = 0;

  mgpu_scene_desc desc() const {
    mgpu_scene_desc d;
    memset(&d, 0, sizeof(d));
    d.ntri = ntri;
    d.tri_v = v.data();
    d.tri_n = n.empty() ? nullptr : n.data();
    d.tri_mat = mat.data();
    d.tri_light = light.empty() ? nullptr : light.data();
    d.tri_flags = flags.empty() ? nullptr : flags.data();
    d.nmat = nmat;
    d.materials = mats.data();
    d.nlight = nlight;
    d.lights = lights.empty() ? nullptr : lights.data();
    d.light_ext = light_ext.empty() ? nullptr : light_ext.data();
    d.tri_uv = uv.empty() ? nullptr : uv.data();
    d.ntex = (int32_t)tex.size();
    d.textures = tex.empty() ? nullptr : tex.data();
    d.background_tex = bg_tex;
    for (int k = 0; k < 3; ++k) d.background_le[k] = bg_le[k];
    d.nsphere = (int32_t)sph_mat.size();
    d.spheres = sph.empty() ? nullptr : sph.data();
    d.sphere_mat = sph_mat.empty() ? nullptr : sph_mat.data();
    d.sphere_light = sph_light.empty() ? nullptr : sph_light.data();
    return d;
  }
};

struct SrvJob {
  int64_t id = 0;
  int32_t scene = 0;
  mgpu_render_params p{};
  int32_t max_spp = 1;
  double target = 0.0;
  double arrival = NAN, admit = NAN, done = NAN;
  int state = MGPU_JOB_QUEUED;
  mgpu_film *film = nullptr;
  int32_t spp_done = 0, next_ckpt = 0;
  int reached = 0;
  double rmse = NAN;
  uint64_t paths = 0;
  uint64_t last_served = 0;
  std::string error;

  uint64_t pixels() const { return (uint64_t)p.width * (uint64_t)p.height; }
  uint64_t film_bytes() const { return pixels() * 32u; }
};

}  // namespace

struct mgpu_server {
  mgpu_server_params p{};
  std::chrono::steady_clock::time_point t0;
  std::vector<std::unique_ptr<SrvScene>> scenes;  // guarded by mu (build threads index it)
  std::vector<std::unique_ptr<SrvJob>> jobs;      // by id
  std::vector<int64_t> queue;                     // queued job ids by (arrival, id)
  std::vector<int64_t> active;                    // active job ids in admission order
  mgpu_batch *batch = nullptr;
  uint64_t resident = 0, peak = 0, scene_bytes = 0, film_bytes = 0;
  uint64_t paths = 0, ticks = 0, admitted = 0, finished = 0, failed = 0, evictions = 0, uploads = 0, builds = 0;
  double render_s = 0.0;
  std::mutex mu;
  std::condition_variable cv;
  std::vector<int32_t> build_q;
  std::vector<std::thread> workers;
  bool stop = false;
  int building = 0;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

using mgpu::fail;

void build_worker(mgpu_server *s) {
  for (;;) {
    SrvScene *sc = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] { return s->stop || !s->build_q.empty(); });
      if (s->stop) return;
      const int32_t id = s->build_q.front();
      s->build_q.erase(s->build_q.begin());
      sc = s->scenes[id].get();
    }
    const mgpu_scene_desc d = sc->desc();
    mgpu_accel *acc = nullptr;
    uint64_t bytes = 0;
    int rc = mgpu_accel_build(&d, &s->p.kd, &acc);
    if (rc == MGPU_OK) rc = mgpu_scene_device_bytes(&d, acc, &bytes);
    const std::string err = rc == MGPU_OK ? std::string() : std::string(mgpu_last_error());
    std::lock_guard<std::mutex> lk(s->mu);
    if (rc == MGPU_OK) {
      sc->accel = acc;
      sc->dev_bytes = bytes;
      sc->state = kBuilt;
      ++s->builds;
    } else {
      if (acc) mgpu_accel_destroy(acc);
      sc->state = kBuildFailed;
      sc->error = err;
    }
    --s->building;
  }
}

// starts the background build of a scene that has none (caller holds no lock)
void request_build(mgpu_server *s, int32_t scene) {
  std::lock_guard<std::mutex> lk(s->mu);
  SrvScene *sc = s->scenes[scene].get();
  if (sc->state != kIdle) return;
  sc->state = kBuilding;
  ++s->building;
  s->build_q.push_back(scene);
  s->cv.notify_one();
}

int scene_state(mgpu_server *s, SrvScene *sc) {
  std::lock_guard<std::mutex> lk(s->mu);
  return sc->state;
}

void account(mgpu_server *s) {
  s->resident = s->scene_bytes + s->film_bytes;
  s->peak = std::max(s->peak, s->resident);
}

// frees idle resident scenes, least recently used first, until `need` more bytes fit
void evict_idle(mgpu_server *s, uint64_t need, int32_t keep) {
  while (s->resident + need > s->p.hbm_budget) {
    SrvScene *victim = nullptr;
    for (size_t i = 0; i < s->scenes.size(); ++i) {
      SrvScene *sc = s->scenes[i].get();
      if ((int32_t)i == keep || !sc->dev || sc->active > 0) continue;
      if (!victim || sc->last_use < victim->last_use) victim = sc;
    }
    if (!victim) return;
    mgpu_scene_destroy(victim->dev);
    victim->dev = nullptr;
    s->scene_bytes -= victim->dev_bytes;
    ++s->evictions;
    account(s);
  }
}

void finish(mgpu_server *s, SrvJob *j, int state, double t) {
  j->state = state;
  j->done = t;
  if (state == MGPU_JOB_DONE) ++s->finished;
  else ++s->failed;
  auto it = std::find(s->active.begin(), s->active.end(), j->id);
  if (it != s->active.end()) {
    s->active.erase(it);
    s->scenes[j->scene]->active -= 1;
  }
}

void fail_job(mgpu_server *s, SrvJob *j, const std::string &why, double t) {
  j->error = why;
  if (j->film) {
    mgpu_film_destroy(j->film);
    j->film = nullptr;
    s->film_bytes -= j->film_bytes();
    account(s);
  }
  finish(s, j, MGPU_JOB_FAILED, t);
}

// Admission in arrival order (see the header).
int admit(mgpu_server *s, void *stream, double now) {
  for (size_t qi = 0; qi < s->queue.size();) {
    if ((int32_t)s->active.size() >= s->p.max_active) break;
    SrvJob *j = s->jobs[s->queue[qi]].get();
    if (j->arrival > now) break;
    SrvScene *sc = s->scenes[j->scene].get();
    const int st = scene_state(s, sc);
    if (st == kIdle || st == kBuilding) {
      if (st == kIdle) request_build(s, j->scene);
      ++qi;
      continue;
    }
    if (st == kBuildFailed) {
      s->queue.erase(s->queue.begin() + qi);
      fail_job(s, j, "kd-tree build failed: " + sc->error, now);
      continue;
    }
    const uint64_t need = j->film_bytes() + (sc->dev ? 0 : sc->dev_bytes);
    if (need > s->p.hbm_budget) {
      s->queue.erase(s->queue.begin() + qi);
      fail_job(s, j, "film and scene exceed the whole memory budget", now);
      continue;
    }
    if (s->resident + need > s->p.hbm_budget) evict_idle(s, need, j->scene);
    if (s->resident + need > s->p.hbm_budget) break;  // wait for running jobs to free memory
    if (!sc->dev) {
      const mgpu_scene_desc d = sc->desc();
      int rc = mgpu_scene_create(&d, sc->accel, stream, &sc->dev);
      if (rc == MGPU_E_NOMEM) break;
      if (rc != MGPU_OK) {
        s->queue.erase(s->queue.begin() + qi);
        fail_job(s, j, std::string("scene upload failed: ") + mgpu_last_error(), now);
        continue;
      }
      s->scene_bytes += sc->dev_bytes;
      ++s->uploads;
      account(s);
    }
    int rc = mgpu_film_create(j->p.width, j->p.height, stream, &j->film);
    if (rc == MGPU_E_NOMEM) break;
    if (rc != MGPU_OK) {
      s->queue.erase(s->queue.begin() + qi);
      fail_job(s, j, std::string("film allocation failed: ") + mgpu_last_error(), now);
      continue;
    }
    s->film_bytes += j->film_bytes();
    account(s);
    j->state = MGPU_JOB_ACTIVE;
    j->admit = now;
    j->next_ckpt = std::min(j->p.spp, j->max_spp);
    sc->active += 1;
    sc->last_use = s->ticks;
    s->active.push_back(j->id);
    ++s->admitted;
    s->queue.erase(s->queue.begin() + qi);
  }
  return MGPU_OK;
}

struct Pass {
  SrvJob *job;
  int32_t samples;
};

// The tick's passes: one sample per job (least recently served first), then the rest of the
// path budget oldest job first, never past a job's next checkpoint.
void plan(mgpu_server *s, std::vector<Pass> &out) {
  out.clear();
  std::vector<SrvJob *> act;
  for (int64_t id : s->active) act.push_back(s->jobs[id].get());
  std::vector<int32_t> k(act.size(), 0);
  int64_t left = s->p.tick_paths;
  std::vector<size_t> order(act.size());
  for (size_t i = 0; i < act.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return act[a]->last_served < act[b]->last_served; });
  bool any = false;
  if (s->p.policy == MGPU_SERVE_FAIR) {
    for (size_t i : order) {
      const int64_t px = (int64_t)act[i]->pixels();
      if (px <= left || !any) {
        k[i] = 1;
        left -= px;
        any = true;
      }
    }
  } else if (!act.empty()) {
    // the oldest (or least recently served) job always advances, even when one sample exceeds
    // the tick
    const size_t first = s->p.policy == MGPU_SERVE_ROTATE ? order[0] : 0;
    k[first] = 1;
    left -= (int64_t)act[first]->pixels();
  }
  if (s->p.policy == MGPU_SERVE_ROTATE) {
    // whole passes in least-recently-served order
    for (size_t i : order) {
      if (left <= 0) break;
      const int64_t px = (int64_t)act[i]->pixels();
      const int64_t room = act[i]->next_ckpt - act[i]->spp_done - k[i];
      const int64_t more = std::min<int64_t>(room, left / px);
      if (more > 0) {
        k[i] += (int32_t)more;
        left -= more * px;
      }
    }
  }
  for (size_t i = 0; i < act.size() && left > 0; ++i) {
    const int64_t px = (int64_t)act[i]->pixels();
    const int64_t room = act[i]->next_ckpt - act[i]->spp_done - k[i];
    const int64_t more = std::min<int64_t>(room, left / px);
    if (more > 0) {
      k[i] += (int32_t)more;
      left -= more * px;
    }
  }
  for (size_t i = 0; i < act.size(); ++i)
    if (k[i] > 0) out.push_back({act[i], k[i]});
  // passes of one scene next to each other: a wave then touches fewer trees (L2 reuse)
  std::stable_sort(out.begin(), out.end(), [](const Pass &a, const Pass &b) { return a.job->scene < b.job->scene; });
}

}  // namespace

extern "C" {

int mgpu_server_create(const mgpu_server_params *params, mgpu_server **out) {
  if (!params || !out) return fail(MGPU_E_INVALID, "mgpu_server_create: null argument");
  if (params->tick_paths < 0 || params->max_active < 0 || params->wave_paths < 0 || params->build_threads < 0)
    return fail(MGPU_E_INVALID, "mgpu_server_create: negative parameter");
  if (params->policy != MGPU_SERVE_FAIR && params->policy != MGPU_SERVE_OLDEST && params->policy != MGPU_SERVE_ROTATE)
    return fail(MGPU_E_INVALID, "mgpu_server_create: unknown policy");
  mgpu_server *s = new (std::nothrow) mgpu_server();
  if (!s) return fail(MGPU_E_NOMEM, "mgpu_server_create: out of host memory");
  s->p = *params;
  if (s->p.hbm_budget == 0) s->p.hbm_budget = 120000000000ull;
  if (s->p.tick_paths == 0) s->p.tick_paths = (int64_t)1 << 26;
  if (s->p.max_active == 0) s->p.max_active = 256;
  if (s->p.build_threads == 0) s->p.build_threads = 2;
  s->t0 = std::chrono::steady_clock::now();
  int rc = mgpu_batch_create(&s->batch);
  if (rc != MGPU_OK) {
    delete s;
    return rc;
  }
  try {
    for (int i = 0; i < s->p.build_threads; ++i) s->workers.emplace_back(build_worker, s);
  } catch (...) {
    mgpu_server_destroy(s);
    return fail(MGPU_E_NOMEM, "mgpu_server_create: cannot start build threads");
  }
  *out = s;
  return MGPU_OK;
}

int mgpu_server_destroy(mgpu_server *s) {
  if (!s) return MGPU_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  for (auto &t : s->workers) t.join();
  for (auto &j : s->jobs)
    if (j->film) mgpu_film_destroy(j->film);
  for (auto &sc : s->scenes) {
    if (sc->dev) mgpu_scene_destroy(sc->dev);
    if (sc->accel) mgpu_accel_destroy(sc->accel);
  }
  if (s->batch) mgpu_batch_destroy(s->batch);
  delete s;
  return MGPU_OK;
}

double mgpu_server_clock(const mgpu_server *s) { return s ? s->now() : NAN; }

int mgpu_server_add_scene(mgpu_server *s, const mgpu_scene_desc *d, int32_t *scene_id) {
  if (!s || !d || !scene_id) return fail(MGPU_E_INVALID, "mgpu_server_add_scene: null argument");
  if (d->ntri < 0 || (d->ntri > 0 && (!d->tri_v || !d->tri_mat)) || d->nmat <= 0 || !d->materials ||
      d->nlight < 0 || (d->nlight > 0 && !d->lights))
    return fail(MGPU_E_INVALID, "mgpu_server_add_scene: incomplete scene description");
  std::unique_ptr<SrvScene> sc(new (std::nothrow) SrvScene());
  if (!sc) return fail(MGPU_E_NOMEM, "mgpu_server_add_scene: out of host memory");
  const size_t T = (size_t)d->ntri;
  try {
    sc->ntri = d->ntri;
    sc->v.assign(d->tri_v, d->tri_v + 9 * T);
    if (d->tri_n) sc->n.assign(d->tri_n, d->tri_n + 9 * T);
    sc->mat.assign(d->tri_mat, d->tri_mat + T);
    if (d->tri_light) sc->light.assign(d->tri_light, d->tri_light + T);
    if (d->tri_flags) sc->flags.assign(d->tri_flags, d->tri_flags + T);
    sc->nmat = d->nmat;
    sc->mats.assign(d->materials, d->materials + 16 * (size_t)d->nmat);
    sc->nlight = d->nlight;
    if (d->nlight > 0) sc->lights.assign(d->lights, d->lights + 16 * (size_t)d->nlight);
    if (d->nlight > 0 && d->light_ext) sc->light_ext.assign(d->light_ext, d->light_ext + 16 * (size_t)d->nlight);
    if (d->tri_uv) sc->uv.assign(d->tri_uv, d->tri_uv + 6 * T);
    if (d->ntex < 0 || (d->ntex > 0 && !d->textures))
      return fail(MGPU_E_INVALID, "mgpu_server_add_scene: bad textures");
    for (int32_t i = 0; i < d->ntex; ++i) {
      mgpu_texture t = d->textures[i];
      if (t.width <= 0 || t.height <= 0 || !t.rgb)
        return fail(MGPU_E_INVALID, "mgpu_server_add_scene: bad texture " + std::to_string(i));
      sc->tex_rgb.emplace_back(t.rgb, t.rgb + (size_t)t.width * t.height * 3);
      sc->tex.push_back(t);
    }
    for (int32_t i = 0; i < d->ntex; ++i) sc->tex[i].rgb = sc->tex_rgb[i].data();
    sc->bg_tex = d->background_tex;
    for (int k = 0; k < 3; ++k) sc->bg_le[k] = d->background_le[k];
    if (d->nsphere < 0 || (d->nsphere > 0 && (!d->spheres || !d->sphere_mat)))
      return fail(MGPU_E_INVALID, "mgpu_server_add_scene: bad spheres");
    if (d->nsphere > 0) {
      sc->sph.assign(d->spheres, d->spheres + 8 * (size_t)d->nsphere);
      sc->sph_mat.assign(d->sphere_mat, d->sphere_mat + d->nsphere);
      if (d->sphere_light) sc->sph_light.assign(d->sphere_light, d->sphere_light + d->nsphere);
    }
  } catch (...) {
    return fail(MGPU_E_NOMEM, "mgpu_server_add_scene: out of host memory");
  }
  std::lock_guard<std::mutex> lk(s->mu);
  s->scenes.push_back(std::move(sc));
  *scene_id = (int32_t)s->scenes.size() - 1;
  return MGPU_OK;
}

int mgpu_server_prefetch(mgpu_server *s, int32_t scene_id) {
  if (!s) return fail(MGPU_E_INVALID, "mgpu_server_prefetch: null server");
  size_t nscenes;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    nscenes = s->scenes.size();
  }
  if (scene_id < 0 || (size_t)scene_id >= nscenes) return fail(MGPU_E_INVALID, "mgpu_server_prefetch: unknown scene");
  request_build(s, scene_id);
  return MGPU_OK;
}

int mgpu_server_submit(mgpu_server *s, int32_t scene_id, const mgpu_render_params *params, int32_t max_spp,
                       double target_rmse, double arrival, int64_t *job_id) {
  if (!s || !params || !job_id) return fail(MGPU_E_INVALID, "mgpu_server_submit: null argument");
  size_t nscenes;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    nscenes = s->scenes.size();
  }
  if (scene_id < 0 || (size_t)scene_id >= nscenes) return fail(MGPU_E_INVALID, "mgpu_server_submit: unknown scene");
  if (max_spp <= 0 || params->width <= 0 || params->height <= 0 || params->spp <= 0 ||
      params->no_direct_samples <= 0 || params->max_depth < 0 || params->rr_start_depth < 0 ||
      (int64_t)params->width * params->height > (int64_t)1 << 31 || !(target_rmse == target_rmse))
    return fail(MGPU_E_INVALID, "mgpu_server_submit: bad parameters");
  std::unique_ptr<SrvJob> j(new (std::nothrow) SrvJob());
  if (!j) return fail(MGPU_E_NOMEM, "mgpu_server_submit: out of host memory");
  j->id = (int64_t)s->jobs.size();
  j->scene = scene_id;
  j->p = *params;
  j->p.sample_begin = 0;
  j->p.sample_count = 0;
  j->p.wave_paths = 0;
  j->max_spp = max_spp;
  j->target = target_rmse;
  j->arrival = arrival < 0 ? s->now() : arrival;
  const int64_t id = j->id;
  const double a = j->arrival;
  s->jobs.push_back(std::move(j));
  auto pos = std::upper_bound(s->queue.begin(), s->queue.end(), a,
                              [&](double t, int64_t q) { return t < s->jobs[q]->arrival; });
  s->queue.insert(pos, id);
  request_build(s, scene_id);
  *job_id = id;
  return MGPU_OK;
}

int mgpu_server_step(mgpu_server *s, void *stream, int32_t *unfinished) {
  if (!s) return fail(MGPU_E_INVALID, "mgpu_server_step: null server");
  int rc = admit(s, stream, s->now());
  if (rc != MGPU_OK) return rc;
  std::vector<Pass> passes;
  plan(s, passes);
  if (!passes.empty()) {
    mgpu_batch_clear(s->batch);
    mgpu_batch_set(s->batch, s->p.wave_paths, s->p.use_graph);
    std::vector<Pass> ok;
    for (const Pass &ps : passes) {
      SrvJob *j = ps.job;
      mgpu_render_params p = j->p;
      p.sample_begin = j->spp_done;
      p.sample_count = ps.samples;
      if (mgpu_batch_add(s->batch, s->scenes[j->scene]->dev, &p, j->film) != MGPU_OK) {
        fail_job(s, j, std::string("bad render parameters: ") + mgpu_last_error(), s->now());
        continue;
      }
      ok.push_back(ps);
    }
    const double ta = s->now();
    rc = mgpu_batch_render(s->batch, stream);
    if (rc != MGPU_OK) return rc;
    std::vector<SrvJob *> ck;
    std::vector<mgpu_film *> films;
    for (const Pass &ps : ok) {
      SrvJob *j = ps.job;
      j->spp_done += ps.samples;
      j->paths += j->pixels() * (uint64_t)ps.samples;
      j->last_served = s->ticks + 1;
      s->paths += j->pixels() * (uint64_t)ps.samples;
      s->scenes[j->scene]->last_use = s->ticks + 1;
      if (j->spp_done >= j->next_ckpt) {
        ck.push_back(j);
        films.push_back(j->film);
      }
    }
    std::vector<double> err(ck.size());
    if (!ck.empty()) {
      rc = mgpu_film_error(films.data(), (int32_t)films.size(), err.data(), stream);
    } else {
      cudaError_t e = cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
      rc = e == cudaSuccess ? MGPU_OK : fail(MGPU_E_CUDA, std::string("mgpu_server_step: ") + cudaGetErrorString(e));
    }
    if (rc != MGPU_OK) return rc;
    const double tb = s->now();
    s->render_s += tb - ta;
    ++s->ticks;
    for (size_t i = 0; i < ck.size(); ++i) {
      SrvJob *j = ck[i];
      j->rmse = err[i];
      if (j->target > 0.0 && err[i] <= j->target) {
        j->reached = 1;
        finish(s, j, MGPU_JOB_DONE, tb);
      } else if (j->spp_done >= j->max_spp) {
        finish(s, j, MGPU_JOB_DONE, tb);
      } else {
        j->next_ckpt = (int32_t)std::min<int64_t>((int64_t)j->next_ckpt * 2, j->max_spp);
      }
    }
  }
  if (unfinished) *unfinished = (int32_t)(s->queue.size() + s->active.size());
  return MGPU_OK;
}

int mgpu_server_job(const mgpu_server *s, int64_t id, mgpu_server_job_info *out) {
  if (!s || !out) return fail(MGPU_E_INVALID, "mgpu_server_job: null argument");
  if (id < 0 || (size_t)id >= s->jobs.size()) return fail(MGPU_E_INVALID, "mgpu_server_job: unknown job");
  const SrvJob *j = s->jobs[id].get();
  out->state = j->state;
  out->scene = j->scene;
  out->spp_done = j->spp_done;
  out->reached_target = j->reached;
  out->rmse = j->rmse;
  out->t_arrival = j->arrival;
  out->t_admit = j->admit;
  out->t_done = j->done;
  out->paths = j->paths;
  return MGPU_OK;
}

int mgpu_server_read(mgpu_server *s, int64_t id, double *out_mean, void *stream) {
  if (!s || !out_mean) return fail(MGPU_E_INVALID, "mgpu_server_read: null argument");
  if (id < 0 || (size_t)id >= s->jobs.size()) return fail(MGPU_E_INVALID, "mgpu_server_read: unknown job");
  SrvJob *j = s->jobs[id].get();
  if (!j->film) return fail(MGPU_E_STATE, "mgpu_server_read: the job has no film (queued, failed or released)");
  return mgpu_film_read(j->film, out_mean, stream);
}

int mgpu_server_release(mgpu_server *s, int64_t id) {
  if (!s) return fail(MGPU_E_INVALID, "mgpu_server_release: null server");
  if (id < 0 || (size_t)id >= s->jobs.size()) return fail(MGPU_E_INVALID, "mgpu_server_release: unknown job");
  SrvJob *j = s->jobs[id].get();
  auto q = std::find(s->queue.begin(), s->queue.end(), id);
  if (q != s->queue.end()) s->queue.erase(q);
  if (j->state == MGPU_JOB_QUEUED || j->state == MGPU_JOB_ACTIVE) {
    fail_job(s, j, "released before it finished", s->now());
    return MGPU_OK;
  }
  if (j->film) {
    mgpu_film_destroy(j->film);
    j->film = nullptr;
    s->film_bytes -= j->film_bytes();
    account(s);
  }
  return MGPU_OK;
}

int mgpu_server_stats_get(const mgpu_server *s, mgpu_server_stats *o) {
  if (!s || !o) return fail(MGPU_E_INVALID, "mgpu_server_stats_get: null argument");
  memset(o, 0, sizeof(*o));
  o->resident_bytes = s->resident;
  o->peak_resident_bytes = s->peak;
  o->scene_bytes = s->scene_bytes;
  o->film_bytes = s->film_bytes;
  o->paths = s->paths;
  o->ticks = s->ticks;
  o->admitted = s->admitted;
  o->finished = s->finished;
  o->failed = s->failed;
  o->evictions = s->evictions;
  o->uploads = s->uploads;
  o->queued = (int32_t)s->queue.size();
  o->active = (int32_t)s->active.size();
  o->render_seconds = s->render_s;
  int resident = 0;
  for (auto &sc : s->scenes) resident += sc->dev ? 1 : 0;
  o->resident_scenes = resident;
  std::lock_guard<std::mutex> lk(const_cast<mgpu_server *>(s)->mu);
  o->builds = s->builds;
  o->building = s->building;
  return MGPU_OK;
}

}  // extern "C"
