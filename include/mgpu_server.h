/*
 * mgpu_server.h -- continuous-batching render service over libmgpu.so.
 *
 * No counterpart in the reference: Milton renders one scene per process, its progressive mode
 * being endless super-sample passes over one image (mlt/src/milton/renderers/generators/
 * SuperSampleGenerator.cpp:54-92).  A server keeps a library of scenes and a queue of render
 * jobs on one device.  A job is one image: a scene, Milton's render parameters (camera,
 * resolution, spp stratification, depth, RR, seed), a cap on samples per pixel and an error
 * target.  Each mgpu_server_step() is one scheduling tick:
 *
 *   1. Admission, in arrival order: a job whose scene's kd-tree is still being built on the
 *      host (a background thread starts the build when the job is submitted) is passed over;
 *      otherwise it is admitted while an active slot is free and its film -- plus its scene,
 *      if that is not resident -- fits the device-memory budget.  Idle resident scenes (no
 *      active job) are evicted least recently used first to make room; a job that still does
 *      not fit stops admission for this tick.  Trees and films stay on the device between
 *      ticks.
 *   2. Rendering: active jobs get sample passes up to the tick's path budget -- under the fair
 *      policy first one sample each, least recently served first, then the rest of the budget
 *      oldest job first; under the oldest-first policy only the latter; under the rotating
 *      policy whole passes (up to the next checkpoint) to the least recently served jobs first
 *      -- never past a job's next checkpoint -- and the passes of all jobs render together in one
 *      batch (mgpu_batch_*: jobs of different scenes share waves; passes are grouped by
 *      scene so that a wave touches few trees).
 *   3. Checkpoints: a job's checkpoints are its sample counts c0 = min(spp, max_spp),
 *      c(k+1) = min(2 c(k), max_spp), spp being its stratification (noSuperSamples).  At each,
 *      mgpu_film_error estimates the film's RMSE; the job finishes when the estimate is at most
 *      target_rmse or max_spp samples are in.
 *
 * A job's film after n samples does not depend on what else shares the device or how its
 * samples were split into passes, and its checkpoints depend on nothing but its own film, so
 * every job finishes with exactly the image (bit for bit) and sample count it gets alone.
 *
 * The budget covers resident scenes and films; a finished job keeps its film (and its share
 * of the budget) until mgpu_server_release, so a client that does not release finished jobs
 * can stall admission.  The render workspace (path state and queues of one wave, shared by
 * all jobs) is allocated once per host thread outside the budget.
 * All calls on one server come from one host thread; times are seconds on the server's clock
 * (a steady clock, zero at creation).
 */
#ifndef MGPU_SERVER_H_
#define MGPU_SERVER_H_

#include "mgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mgpu_server mgpu_server;

typedef struct {
  uint64_t hbm_budget;   /* device bytes for resident scenes and films; 0 = 120e9 */
  int64_t tick_paths;    /* paths rendered per tick over all jobs; 0 = 2^26 */
  int32_t max_active;    /* job slots on the device; 0 = 256 */
  int32_t wave_paths;    /* paths in flight per wave; 0 = automatic */
  int32_t use_graph;     /* capture each tick's launches in one CUDA graph */
  int32_t build_threads; /* background kd-tree builds at once; 0 = 2 */
  mgpu_kd_params kd;     /* kd-tree parameters for every scene (threads 0 = all cores) */
  int32_t policy;        /* MGPU_SERVE_FAIR (0): one sample per active job first, least recently
                            served first, then the rest oldest first; MGPU_SERVE_OLDEST (1): the
                            whole tick oldest job first (fewer jobs and scenes per wave);
                            MGPU_SERVE_ROTATE (2): whole passes, least recently served job first
                            (fewer, larger passes per tick: more samples of a pixel in a wave) */
} mgpu_server_params;

#define MGPU_SERVE_FAIR 0
#define MGPU_SERVE_OLDEST 1
#define MGPU_SERVE_ROTATE 2

#define MGPU_JOB_QUEUED 0
#define MGPU_JOB_ACTIVE 1
#define MGPU_JOB_DONE 2
#define MGPU_JOB_FAILED 3

typedef struct {
  int32_t state;          /* MGPU_JOB_* */
  int32_t scene;
  int32_t spp_done;       /* samples per pixel in the film */
  int32_t reached_target; /* 1: finished with error <= target_rmse; 0: at max_spp or not done */
  double rmse;            /* error estimate at the last checkpoint (NaN before the first) */
  double t_arrival, t_admit, t_done; /* server clock; NaN until the event */
  uint64_t paths;         /* paths rendered for the job */
} mgpu_server_job_info;

typedef struct {
  uint64_t resident_bytes, peak_resident_bytes, scene_bytes, film_bytes;
  uint64_t paths, ticks, admitted, finished, failed, evictions, uploads, builds;
  int32_t queued, active, resident_scenes, building;
  double render_seconds; /* wall time spent in render ticks */
} mgpu_server_stats;

int mgpu_server_create(const mgpu_server_params *params, mgpu_server **out);
/* Waits for background builds, frees every film and scene.                                */
int mgpu_server_destroy(mgpu_server *server);
double mgpu_server_clock(const mgpu_server *server);
/* Copies the scene's arrays (the server owns the copy); returns its index in scene_id.     */
int mgpu_server_add_scene(mgpu_server *server, const mgpu_scene_desc *desc, int32_t *scene_id);
/* Starts the scene's background kd-tree build now instead of at its first submit.          */
int mgpu_server_prefetch(mgpu_server *server, int32_t scene_id);
/* Queues a job.  params: width, height, spp (stratification), camera, depth, RR, seed,
 * stream_id as for mgpu_render; sample_begin, sample_count and wave_paths are ignored.
 * arrival: the request's arrival time on the server clock (< 0 = now); a job is not admitted
 * before it.  target_rmse <= 0 renders to max_spp.                                        */
int mgpu_server_submit(mgpu_server *server, int32_t scene_id, const mgpu_render_params *params, int32_t max_spp,
                       double target_rmse, double arrival, int64_t *job_id);
/* One tick (synchronises with the stream).  unfinished = jobs queued or active after it.   */
int mgpu_server_step(mgpu_server *server, void *stream, int32_t *unfinished);
int mgpu_server_job(const mgpu_server *server, int64_t job_id, mgpu_server_job_info *out);
/* Per-pixel mean of a job's film (width*height*3 doubles), as mgpu_film_read.              */
int mgpu_server_read(mgpu_server *server, int64_t job_id, double *out_mean, void *stream);
/* Frees the job's film (cancelling it if unfinished); its info stays queryable.             */
int mgpu_server_release(mgpu_server *server, int64_t job_id);
int mgpu_server_stats_get(const mgpu_server *server, mgpu_server_stats *out);

#ifdef __cplusplus
}
#endif
#endif /* MGPU_SERVER_H_ */
