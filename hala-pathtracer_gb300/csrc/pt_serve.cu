// pt_serve.cu -- the job server of include/hala_pt.h (pt_server_*):
// continuous batching of render jobs into shared wavefronts.
//
// Two host threads per server:
//   admission  takes queued jobs in arrival order while the head job's
//              estimated device bytes fit the budget and a job slot is free;
//              uploads the scene on the job's own stream, builds its BVH and
//              environment tables (pt_renderer_set_scene/commit) and hands it
//              to the render thread. A job that does not fit waits at the head
//              of the queue, so large jobs are not starved by small ones.
//   render     forms one wavefront at a time from the running jobs of one
//              feature permutation (round robin over permutations), gives each
//              job up to `quantum_paths` paths per turn until the wavefront is
//              full, runs the bounce loop once for all of them, accumulates
//              each job's run of paths into its own images, and tonemaps and
//              retires jobs whose last path is in.
// The device keeps one DevScene record per job slot; the shared-wavefront
// kernels read a path's scene through its slot. A job's path g is always
// initialised from (its scene, g), whatever else shares the wavefront, and its
// paths are accumulated in increasing g, so its images are those of a
// pt_renderer render of the same job.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pt_impl.h"

namespace hpt {
namespace {

using Clock = std::chrono::steady_clock;

// Deep copy of a pt_job_desc: the caller's arrays may go away after submit.
struct JobInput {
  pt_tracer_config cfg{};
  uint32_t frames = 0, camera_index = 0;
  std::vector<std::vector<float>> verts;
  std::vector<std::vector<uint32_t>> idx;
  std::vector<pt_primitive> prims;
  std::vector<pt_material> mats;
  std::vector<pt_light> lights;
  std::vector<pt_camera> cams;
  std::vector<std::vector<float>> tex_px;
  std::vector<pt_texture> texs;
  std::vector<float> env;
  uint32_t env_w = 0, env_h = 0;
  float env_rot = 0.0f, env_intensity = 1.0f, exposure = 0.0f;
  float ground[4] = {0, 0, 0, 1}, sky[4] = {0, 0, 0, 1};
  bool use_cache = false;
  pt_cache_config cache_cfg{};
  pt_scene_desc desc{};

  void copy_from(const pt_job_desc& j) {
    const pt_scene_desc& s = *j.scene;
    cfg = j.config;
    frames = j.frames;
    camera_index = j.camera_index;
    prims.assign(s.primitives, s.primitives + s.num_primitives);
    verts.resize(prims.size());
    idx.resize(prims.size());
    for (size_t i = 0; i < prims.size(); ++i) {
      verts[i].assign(prims[i].vertices, prims[i].vertices + 11 * (size_t)prims[i].num_vertices);
      idx[i].assign(prims[i].indices, prims[i].indices + prims[i].num_indices);
      prims[i].vertices = verts[i].data();
      prims[i].indices = idx[i].data();
    }
    mats.assign(s.materials, s.materials + s.num_materials);
    lights.assign(s.lights, s.lights + s.num_lights);
    cams.assign(s.cameras, s.cameras + s.num_cameras);
    texs.assign(s.textures, s.textures + s.num_textures);
    tex_px.resize(texs.size());
    for (size_t i = 0; i < texs.size(); ++i) {
      if (texs[i].rgba) tex_px[i].assign(texs[i].rgba, texs[i].rgba + 4 * (size_t)texs[i].width * texs[i].height);
      texs[i].rgba = tex_px[i].empty() ? nullptr : tex_px[i].data();
    }
    if (j.env_rgb && j.env_width && j.env_height) {
      env.assign(j.env_rgb, j.env_rgb + 3 * (size_t)j.env_width * j.env_height);
      env_w = j.env_width;
      env_h = j.env_height;
    }
    env_rot = j.env_rotation_deg;
    env_intensity = j.env_intensity;
    exposure = j.exposure_value;
    std::memcpy(ground, j.ground_color, sizeof(ground));
    std::memcpy(sky, j.sky_color, sizeof(sky));
    use_cache = j.cache != nullptr;
    if (use_cache) cache_cfg = *j.cache;
    desc = pt_scene_desc{prims.data(), (uint32_t)prims.size(), mats.data(), (uint32_t)mats.size(),
                         lights.data(), (uint32_t)lights.size(), cams.data(), (uint32_t)cams.size(),
                         texs.data(), (uint32_t)texs.size()};
  }
};

// Job class bit of a job with a radiance cache: such a job never shares a
// wavefront (its passes train its own cache in between); the scheduler
// gives it whole passes through its own renderer, in turn with the shared
// wavefronts of the other jobs.
constexpr uint32_t JOB_CACHE_CLASS = 0x100u;

enum : int { ST_QUEUED = PT_JOB_QUEUED, ST_RUNNING = PT_JOB_RUNNING, ST_DONE = PT_JOB_DONE,
             ST_FAILED = PT_JOB_FAILED, ST_CANCELLED = PT_JOB_CANCELLED };

struct Job {
  uint64_t id = 0;
  std::unique_ptr<JobInput> in;  // until admission
  pt_renderer* r = nullptr;      // device-resident scene and images once admitted
  std::mutex io;                 // held while images are read and while the renderer is freed
  int state = ST_QUEUED;
  pt_status status = PT_OK;
  std::string err;
  uint64_t total = 0, done = 0;
  uint32_t WH = 0;
  uint32_t slot = UINT32_MAX;
  uint32_t features = 0;
  uint64_t est = 0;        // admission estimate, counted in resident bytes while held
  uint64_t image_bytes = 0;
  uint32_t pass_frames = 0;  // frames per turn of a job with a radiance cache
  double t_submit = 0, t_admit = 0, t_done = 0;
  bool cancel = false, release = false, slot_dirty = false;
  bool terminal() const { return state >= ST_DONE; }
};
using JobPtr = std::shared_ptr<Job>;

}  // namespace
}  // namespace hpt

using namespace hpt;

struct pt_server {
  pt_server_config cfg{};
  int device = 0;
  Clock::time_point t0;

  std::mutex mu;
  std::condition_variable cv_admit, cv_render, cv_done;
  bool stop = false, paused = false;
  std::string err;
  std::map<uint64_t, JobPtr> jobs;
  std::deque<JobPtr> queue;
  std::vector<JobPtr> running;  // admission order
  std::vector<uint32_t> free_slots;
  uint32_t admitting = 0;
  uint64_t next_id = 1;
  uint64_t resident = 0;
  uint32_t rr_class = 0;  // round-robin cursor over running jobs
  pt_server_stats st{};

  // render thread only
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint32_t* pinned = nullptr;
  DevScene* h_jobs = nullptr;  // pinned staging of the slot records
  Buf<DevScene> d_jobs;
  Buf<WaveSegment> d_segs;
  WaveSegment* h_segs = nullptr;  // pinned
  uint32_t seg_cap = 0;
  WaveBuffers W;
  Buf<uint32_t> errw;  // traversal error word of every job's scene record (TRAV_ERR_* bits)

  std::thread admit_thr, render_thr;

  double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
};

namespace {

void finish_job(pt_server* s, const JobPtr& j, int state, pt_status status, const std::string& why) {
  // caller holds s->mu
  j->state = state;
  j->status = status;
  j->err = why;
  j->t_done = s->now_ms();
  if (state == ST_DONE) ++s->st.jobs_done;
  else if (state == ST_FAILED) ++s->st.jobs_failed;
  else if (state == ST_CANCELLED) ++s->st.jobs_cancelled;
  if (j->slot != UINT32_MAX) {
    s->free_slots.push_back(j->slot);
    j->slot = UINT32_MAX;
  }
  s->cv_done.notify_all();
  s->cv_admit.notify_all();
}

void destroy_renderer(const JobPtr& j) {
  std::lock_guard<std::mutex> g(j->io);
  if (j->r) pt_renderer_destroy(j->r);
  j->r = nullptr;
}

// Uploads and commits one job (admission thread, no server lock held).
pt_status admit_job(pt_server* s, Job& j, std::string& why) {
  if (s->cfg.fail_admission_of_job && j.id == s->cfg.fail_admission_of_job) {
    why = "injected admission failure: device allocation refused";
    return PT_ERR_OOM;
  }
  JobInput& in = *j.in;
  pt_tracer_config c = in.cfg;
  c.keep_samples = 0;
  // shared wavefronts use the server's buffers; a cached job renders its own passes
  c.wave_paths = in.use_cache ? std::max<uint32_t>(in.cache_cfg.paths_per_pass, 1u << 16) : 1;
  pt_renderer* r = nullptr;
  // uploads and BVH builds of admitted jobs go ahead of the running wavefronts
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  pt_status ps = renderer_create_with_priority(&c, greatest, &r);
  if (ps != PT_OK) {
    why = "renderer creation failed";
    return ps;
  }
  auto bail = [&](pt_status e) {
    why = pt_renderer_last_error(r);
    pt_renderer_destroy(r);
    return e;
  };
  if ((ps = pt_renderer_set_scene(r, &in.desc)) != PT_OK) return bail(ps);
  if (!in.env.empty() && (ps = pt_renderer_set_envmap(r, in.env.data(), in.env_w, in.env_h, in.env_rot)) != PT_OK)
    return bail(ps);
  pt_renderer_set_ground_color(r, in.ground);
  pt_renderer_set_sky_color(r, in.sky);
  pt_renderer_set_env_intensity(r, in.env_intensity);
  pt_renderer_set_exposure_value(r, in.exposure);
  if ((ps = pt_renderer_set_camera_index(r, in.camera_index)) != PT_OK) return bail(ps);
  if ((ps = pt_renderer_commit(r)) != PT_OK) return bail(ps);
  renderer_drop_build_inputs(r);
  j.features = r->features;
  if (in.use_cache) {
    if ((ps = pt_renderer_set_radiance_cache(r, &in.cache_cfg)) != PT_OK) return bail(ps);
    j.features |= JOB_CACHE_CLASS;
    const uint64_t per = std::max<uint32_t>(in.cache_cfg.paths_per_pass, 1u);
    j.pass_frames = (uint32_t)std::max<uint64_t>(1, (per + j.WH - 1) / j.WH);
  }
  j.r = r;
  return PT_OK;
}

void admission_loop(pt_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    while (!s->queue.empty() && s->queue.front()->cancel) {
      JobPtr c = s->queue.front();
      s->queue.pop_front();
      c->in.reset();
      finish_job(s, c, ST_CANCELLED, PT_ERR_CANCELLED, "cancelled while queued");
    }
    bool go = false;
    if (!s->queue.empty()) {
      const JobPtr& h = s->queue.front();
      go = !s->free_slots.empty() && s->resident + h->est <= s->cfg.hbm_budget_bytes;
    }
    if (!go) {
      s->cv_admit.wait(lk);
      continue;
    }
    JobPtr j = s->queue.front();
    s->queue.pop_front();
    j->slot = s->free_slots.back();
    s->free_slots.pop_back();
    s->resident += j->est;
    s->st.peak_resident_bytes = std::max(s->st.peak_resident_bytes, s->resident);
    ++s->admitting;
    lk.unlock();
    std::string why;
    pt_status ps = admit_job(s, *j, why);
    j->in.reset();
    lk.lock();
    --s->admitting;
    if (ps != PT_OK) {
      s->resident -= j->est;
      finish_job(s, j, ST_FAILED, ps, why);
      continue;
    }
    if (j->cancel || s->stop) {
      s->resident -= j->est;
      finish_job(s, j, ST_CANCELLED, PT_ERR_CANCELLED, "cancelled during admission");
      lk.unlock();
      destroy_renderer(j);
      lk.lock();
      continue;
    }
    j->state = ST_RUNNING;
    j->t_admit = s->now_ms();
    j->slot_dirty = true;
    s->running.push_back(j);
    s->cv_render.notify_all();
  }
}

struct Segment {
  JobPtr job;
  uint32_t start, count;
  uint64_t g0;
};

// Picks the next wavefront (caller holds s->mu). Returns false if no running
// job has paths left.
bool plan_wave(pt_server* s, std::vector<Segment>& segs, uint32_t cap) {
  segs.clear();
  const size_t n = s->running.size();
  size_t first = SIZE_MAX;
  for (size_t k = 0; k < n; ++k) {
    size_t i = (s->rr_class + k) % n;
    const JobPtr& j = s->running[i];
    if (!j->cancel && j->done < j->total) {
      first = i;
      break;
    }
  }
  if (first == SIZE_MAX) return false;
  s->rr_class = (uint32_t)((first + 1) % n);
  const uint32_t cls = s->running[first]->features;
  if (cls & JOB_CACHE_CLASS) {  // a pass of its own
    const JobPtr& j = s->running[first];
    const uint64_t frames = std::min<uint64_t>(j->pass_frames, (j->total - j->done) / j->WH);
    segs.push_back(Segment{j, 0, (uint32_t)(frames * j->WH), j->done});
    return true;
  }
  std::vector<size_t> members;
  for (size_t k = 0; k < n; ++k) {
    size_t i = (first + k) % n;
    const JobPtr& j = s->running[i];
    if (!j->cancel && j->done < j->total && j->features == cls && !(cls & JOB_CACHE_CLASS)) members.push_back(i);
  }
  std::vector<uint64_t> take(members.size(), 0);
  const uint64_t q = std::max<uint32_t>(s->cfg.quantum_paths, 1);
  uint64_t room = cap;
  bool progress = true;
  while (room > 0 && progress) {
    progress = false;
    for (size_t m = 0; m < members.size() && room > 0; ++m) {
      const JobPtr& j = s->running[members[m]];
      uint64_t left = j->total - j->done - take[m];
      uint64_t t = std::min<uint64_t>(std::min<uint64_t>(q, left), room);
      if (t == 0) continue;
      take[m] += t;
      room -= t;
      progress = true;
    }
  }
  uint32_t start = 0;
  for (size_t m = 0; m < members.size(); ++m) {
    if (!take[m]) continue;
    const JobPtr& j = s->running[members[m]];
    segs.push_back(Segment{j, start, (uint32_t)take[m], j->done});
    start += (uint32_t)take[m];
  }
  return true;
}

// Runs one wavefront on the server stream (render thread, no lock held).
cudaError_t run_wave(pt_server* s, std::vector<Segment>& segs, uint32_t total, uint64_t* launches, bool* timed_out,
                     uint64_t rays[2], float* ms, uint32_t* trav_err) {
  cudaError_t e;
  cudaStream_t st = s->stream;
  const bool med = (segs[0].job->features & PT_FEATURE_MEDIUM) != 0;
  if ((e = s->W.ensure(std::max(total, s->cfg.wave_paths), med, true)) != cudaSuccess) return e;
  s->W.P.jobs = s->d_jobs.p;
  if (segs.size() > s->seg_cap) {
    uint32_t c = (uint32_t)std::max<size_t>(segs.size(), 2 * s->seg_cap);
    if (s->h_segs) cudaFreeHost(s->h_segs);
    s->h_segs = nullptr;
    s->seg_cap = 0;
    if ((e = cudaMallocHost(&s->h_segs, c * sizeof(WaveSegment))) != cudaSuccess) return e;
    if ((e = s->d_segs.ensure(c)) != cudaSuccess) return e;
    s->seg_cap = c;
  }
  for (Segment& g : segs) {
    Job& j = *g.job;
    if (j.slot_dirty) {
      s->h_jobs[j.slot] = j.r->view;
      s->h_jobs[j.slot].err = s->errw.p;
      if ((e = cudaMemcpyAsync(s->d_jobs.p + j.slot, s->h_jobs + j.slot, sizeof(DevScene), cudaMemcpyHostToDevice,
                               st)) != cudaSuccess)
        return e;
      j.slot_dirty = false;
    }
  }
  for (size_t k = 0; k < segs.size(); ++k)
    s->h_segs[k] = WaveSegment{segs[k].job->slot, segs[k].start, segs[k].count, 0u, segs[k].g0};
  if ((e = cudaMemcpyAsync(s->d_segs.p, s->h_segs, segs.size() * sizeof(WaveSegment), cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return e;
  if ((e = cudaMemsetAsync(s->W.rays.p, 0, 4 * sizeof(unsigned long long), st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(s->errw.p, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
  if ((e = cudaEventRecord(s->ev0, st)) != cudaSuccess) return e;
  launch_camera_multi(s->W.P, s->d_segs.p, (uint32_t)segs.size(), total, s->W.q_a.p,
                      s->W.counters.p + Q_COUNT + Q_NEXT, st);
  uint32_t max_depth = 0;
  for (Segment& g : segs) max_depth = std::max(max_depth, g.job->r->cfg.max_depth);
  // The shared-wavefront kernels read each path's scene from the slot table;
  // the scene record they take by value only carries the feature set, so
  // the bounce graph captured for one feature set serves every wavefront of it.
  DevScene S;
  std::memset(&S, 0, sizeof(S));
  S.features = segs[0].job->r->view.features;
  BounceLoop L;
  if ((e = run_bounces(S, s->W, total, max_depth, L, s->pinned, st)) != cudaSuccess) return e;
  *launches = L.launches;
  *timed_out = L.timed_out;
  if (L.timed_out) return cudaSuccess;
  for (Segment& g : segs) {
    pt_renderer* r = g.job->r;
    launch_accumulate(s->W.P, g.g0, g.count, g.job->WH, r->accum.p, r->albedo.p, r->normal.p, nullptr, nullptr, 0,
                      st, g.start);
    if (g.g0 + g.count == g.job->total)
      launch_finalize(r->accum.p, r->final_img.p, g.job->WH, r->exposure, r->cfg.enable_tonemap, r->cfg.enable_aces,
                      r->cfg.use_simple_aces, st);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(s->ev1, st)) != cudaSuccess) return e;
  unsigned long long* hr = reinterpret_cast<unsigned long long*>(s->pinned + 16);
  if ((e = cudaMemcpyAsync(hr, s->W.rays.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st)) !=
      cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(s->pinned + 24, s->errw.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  rays[0] = hr[0];
  rays[1] = hr[1];
  *trav_err = s->pinned[24];
  cudaEventElapsedTime(ms, s->ev0, s->ev1);
  return cudaSuccess;
}

void render_loop(pt_server* s) {
  cudaSetDevice(s->device);
  std::vector<Segment> segs;
  std::vector<JobPtr> dead;
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    // retire cancelled running jobs (between wavefronts nothing of theirs is in flight)
    for (size_t i = 0; i < s->running.size();) {
      JobPtr j = s->running[i];
      if (j->cancel) {
        s->running.erase(s->running.begin() + i);
        s->resident -= j->est;
        finish_job(s, j, ST_CANCELLED, PT_ERR_CANCELLED, "cancelled while running");
        dead.push_back(j);
      } else {
        ++i;
      }
    }
    if (!dead.empty()) {
      lk.unlock();
      for (JobPtr& j : dead) destroy_renderer(j);
      dead.clear();
      lk.lock();
      continue;
    }
    if (s->paused || !plan_wave(s, segs, s->cfg.wave_paths)) {
      s->cv_render.wait(lk);
      continue;
    }
    uint32_t total = 0;
    for (const Segment& g : segs) total += g.count;
    if (segs[0].job->features & JOB_CACHE_CLASS) {
      JobPtr j = segs[0].job;
      const uint32_t frames = segs[0].count / j->WH;
      lk.unlock();
      const pt_status ps = pt_renderer_render(j->r, frames);
      const pt_stats rs = j->r->stats;
      const std::string why = ps == PT_OK ? std::string() : std::string(pt_renderer_last_error(j->r));
      lk.lock();
      ++s->st.wavefronts;
      if (ps != PT_OK) {
        auto it = std::find(s->running.begin(), s->running.end(), j);
        if (it != s->running.end()) s->running.erase(it);
        s->resident -= j->est;
        finish_job(s, j, ST_FAILED, ps, why);
        dead.push_back(j);
        continue;
      }
      s->st.paths += rs.paths;
      s->st.closest_rays += rs.closest_rays;
      s->st.shadow_rays += rs.shadow_rays;
      s->st.busy_ms += rs.render_ms;
      s->st.kernel_launches += rs.kernel_launches;
      j->done += (uint64_t)frames * j->WH;
      if (j->done == j->total) {
        auto it = std::find(s->running.begin(), s->running.end(), j);
        if (it != s->running.end()) s->running.erase(it);
        s->resident -= j->est - j->image_bytes;
        j->est = j->image_bytes;
        finish_job(s, j, ST_DONE, PT_OK, "");
        lk.unlock();
        {
          std::lock_guard<std::mutex> g2(j->io);
          pt_renderer_set_radiance_cache(j->r, nullptr);
          j->r->W.release();
          renderer_drop_scene(j->r);
        }
        lk.lock();
      }
      continue;
    }
    lk.unlock();
    uint64_t bounce_launches = 0;
    bool timed_out = false;
    uint64_t rays[2] = {0, 0};
    float ms = 0.0f;
    uint32_t trav_err = 0;
    cudaError_t e = run_wave(s, segs, total, &bounce_launches, &timed_out, rays, &ms, &trav_err);
    lk.lock();
    ++s->st.wavefronts;
    if (e != cudaSuccess || timed_out || trav_err) {
      const std::string why = e != cudaSuccess ? std::string("CUDA error in a wavefront: ") + cudaGetErrorString(e)
                              : timed_out      ? std::string("paths still alive after the bounce cap")
                                               : std::string("BVH traversal exceeded its stack or visit limit");
      const pt_status code = e != cudaSuccess ? PT_ERR_CUDA : timed_out ? PT_ERR_TIMEOUT : PT_ERR_TRAVERSAL;
      for (Segment& g : segs) {
        JobPtr j = g.job;
        auto it = std::find(s->running.begin(), s->running.end(), j);
        if (it != s->running.end()) s->running.erase(it);
        s->resident -= j->est;
        finish_job(s, j, ST_FAILED, code, why);
        dead.push_back(j);
      }
      continue;
    }
    s->st.paths += total;
    s->st.closest_rays += rays[0];
    s->st.shadow_rays += rays[1];
    s->st.busy_ms += ms;
    s->st.kernel_launches += 1 + bounce_launches;  // camera + bounces
    for (Segment& g : segs) {
      JobPtr j = g.job;
      j->done += g.count;
      ++s->st.kernel_launches;  // accumulate
      if (j->done == j->total) {
        ++s->st.kernel_launches;  // finalize
        auto it = std::find(s->running.begin(), s->running.end(), j);
        if (it != s->running.end()) s->running.erase(it);
        // only the images stay resident until release
        s->resident -= j->est - j->image_bytes;
        j->est = j->image_bytes;
        finish_job(s, j, ST_DONE, PT_OK, "");
        lk.unlock();
        {
          std::lock_guard<std::mutex> g2(j->io);
          renderer_drop_scene(j->r);
        }
        lk.lock();
      }
    }
  }
  // shutdown: whatever still runs is cancelled
  for (JobPtr& j : s->running) {
    s->resident -= j->est;
    finish_job(s, j, ST_CANCELLED, PT_ERR_CANCELLED, "server destroyed");
  }
  s->running.clear();
}

pt_status srv_fail(pt_server* s, pt_status st, const std::string& m) {
  std::lock_guard<std::mutex> g(s->mu);
  s->err = m;
  return st;
}

JobPtr find_job(pt_server* s, uint64_t id) {
  auto it = s->jobs.find(id);
  return it == s->jobs.end() ? nullptr : it->second;
}

}  // namespace

// host_exception_status for the server handle, whose last-error text is
// guarded by its mutex (an exception thrown under the lock has released it).
static pt_status server_exception_status(const pt_server* s) noexcept {
  std::string why;
  const pt_status st = host_exception_status(&why);
  if (s) {
    try {
      pt_server* m = const_cast<pt_server*>(s);
      std::lock_guard<std::mutex> g(m->mu);
      m->err = why;
    } catch (...) {
    }
  }
  return st;
}

extern "C" {

pt_status pt_server_create(const pt_server_config* cfg, pt_server** out) try {
  if (!out) return PT_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PT_ERR_CUDA;
  pt_server* s = new pt_server();
  if (cfg) s->cfg = *cfg;
  cudaGetDevice(&s->device);
  if (s->cfg.max_jobs == 0) s->cfg.max_jobs = 64;
  if (s->cfg.wave_paths == 0) s->cfg.wave_paths = 1u << 25;
  if (s->cfg.quantum_paths == 0) s->cfg.quantum_paths = 1u << 18;
  if (s->cfg.hbm_budget_bytes == 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    const uint64_t wave = WaveBuffers::bytes_per_path(true, true) * s->cfg.wave_paths;
    s->cfg.hbm_budget_bytes = fr > wave ? (uint64_t)((fr - wave) * 0.8) : 0;
  }
  s->t0 = Clock::now();
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess ||
      cudaMallocHost(&s->pinned, 256) != cudaSuccess ||
      cudaMallocHost(&s->h_jobs, s->cfg.max_jobs * sizeof(DevScene)) != cudaSuccess ||
      s->d_jobs.ensure(s->cfg.max_jobs) != cudaSuccess || s->errw.ensure(1) != cudaSuccess) {
    pt_server_destroy(s);
    return PT_ERR_CUDA;
  }
  for (uint32_t i = s->cfg.max_jobs; i-- > 0;) s->free_slots.push_back(i);
  s->admit_thr = std::thread(admission_loop, s);
  s->render_thr = std::thread(render_loop, s);
  *out = s;
  return PT_OK;
} catch (...) {
  return host_exception_status(nullptr);
}

void pt_server_destroy(pt_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    for (auto& kv : s->jobs) kv.second->cancel = true;
    s->cv_admit.notify_all();
    s->cv_render.notify_all();
  }
  if (s->admit_thr.joinable()) s->admit_thr.join();
  if (s->render_thr.joinable()) s->render_thr.join();
  for (auto& kv : s->jobs) destroy_renderer(kv.second);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->pinned) cudaFreeHost(s->pinned);
  if (s->h_jobs) cudaFreeHost(s->h_jobs);
  if (s->h_segs) cudaFreeHost(s->h_segs);
  cudaStream_t st = s->stream;
  delete s;
  if (st) cudaStreamDestroy(st);
}

const char* pt_server_last_error(const pt_server* s) {
  static thread_local std::string copy;
  if (!s) return "null server";
  std::lock_guard<std::mutex> g(const_cast<pt_server*>(s)->mu);
  copy = s->err;
  return copy.c_str();
}

pt_status pt_server_submit(pt_server* s, const pt_job_desc* jd, uint64_t* job_id) try {
  if (!s || !jd || !job_id) return PT_ERR_INVALID_ARG;
  std::string why;
  pt_status v = validate_scene_desc(jd->scene, &why);
  if (v == PT_OK) v = validate_tracer_config(&jd->config, &why);
  if (v == PT_OK && jd->frames == 0) v = PT_ERR_INVALID_ARG, why = "frames must be positive";
  if (v == PT_OK && jd->camera_index >= jd->scene->num_cameras) v = PT_ERR_INVALID_ARG, why = "camera index out of range";
  if (v == PT_OK && jd->env_rgb && (jd->env_width == 0 || jd->env_height == 0))
    v = PT_ERR_INVALID_ARG, why = "environment map without a size";
  if (v == PT_OK && jd->cache) {
    for (uint32_t i = 0; i < jd->scene->num_materials; ++i)
      if (jd->scene->materials[i].medium.type != PT_MEDIUM_NONE) {
        v = PT_ERR_UNSUPPORTED;
        why = "the radiance cache does not support participating media";
        break;
      }
  }
  const uint32_t ew = jd->env_rgb ? jd->env_width : 0, eh = jd->env_rgb ? jd->env_height : 0;
  uint64_t est = 0;
  if (v == PT_OK) {
    est = renderer_estimate_bytes(jd->scene, jd->config.width, jd->config.height, ew, eh);
    if (jd->cache) {
      // the cache (hash table with its Adam state, MLP), its per-path buffers
      // and the job's own wavefront of paths_per_pass paths
      const uint32_t log2t = jd->cache->log2_table_size ? jd->cache->log2_table_size : 19;
      const uint64_t per = std::max<uint32_t>(jd->cache->paths_per_pass ? jd->cache->paths_per_pass : 1u << 20,
                                              1u << 16);
      const uint64_t batch = jd->cache->batch_size ? jd->cache->batch_size : 1u << 16;
      est += 16ull * (1ull << log2t) * 2 * 18 + per * (WaveBuffers::bytes_per_path(false, false) + 240) +
             batch * 64 * 6 * 2 * 2 + (16u << 20);
    }
    if (est > s->cfg.hbm_budget_bytes) {
      v = PT_ERR_OOM;
      why = "job needs about " + std::to_string(est >> 20) + " MiB, more than the whole budget of " +
            std::to_string(s->cfg.hbm_budget_bytes >> 20) + " MiB";
    }
  }
  if (v != PT_OK) {
    std::lock_guard<std::mutex> g(s->mu);
    ++s->st.jobs_rejected;
    s->err = why;
    return v;
  }
  JobPtr j = std::make_shared<Job>();
  j->in.reset(new JobInput());
  j->in->copy_from(*jd);
  j->WH = jd->config.width * jd->config.height;
  // render() stops at max_samples frames (src/config/tracer.rs:25)
  uint64_t frames = jd->frames;
  if (jd->config.max_samples > 0) frames = std::min<uint64_t>(frames, jd->config.max_samples);
  j->total = (uint64_t)j->WH * frames;
  j->est = est;
  j->image_bytes = (uint64_t)j->WH * (3 * 16 + 4);
  std::lock_guard<std::mutex> g(s->mu);
  j->id = s->next_id++;
  j->t_submit = s->now_ms();
  s->jobs[j->id] = j;
  s->queue.push_back(j);
  ++s->st.jobs_submitted;
  *job_id = j->id;
  s->cv_admit.notify_all();
  return PT_OK;
} catch (...) {
  return server_exception_status(s);
}

pt_status pt_server_poll(pt_server* s, uint64_t id, pt_job_info* info) try {
  if (!s || !info) return PT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  JobPtr j = find_job(s, id);
  if (!j) {
    s->err = "unknown job id";
    return PT_ERR_INVALID_ARG;
  }
  std::memset(info, 0, sizeof(*info));
  info->id = j->id;
  info->state = j->state;
  info->status = j->status;
  info->paths_total = j->total;
  info->paths_done = j->done;
  info->device_bytes = j->est;
  info->submit_ms = j->t_submit;
  info->admit_ms = j->t_admit;
  info->done_ms = j->t_done;
  std::strncpy(info->error, j->err.c_str(), sizeof(info->error) - 1);
  return PT_OK;
} catch (...) {
  return server_exception_status(s);
}

pt_status pt_server_wait(pt_server* s, uint64_t id, uint32_t timeout_ms) try {
  if (!s) return PT_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  JobPtr j = find_job(s, id);
  if (!j) {
    s->err = "unknown job id";
    return PT_ERR_INVALID_ARG;
  }
  auto pred = [&] { return j->terminal(); };
  if (timeout_ms == 0) {
    s->cv_done.wait(lk, pred);
    return PT_OK;
  }
  if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return PT_ERR_TIMEOUT;
  return PT_OK;
} catch (...) {
  return server_exception_status(s);
}

pt_status pt_server_read_image(pt_server* s, uint64_t id, pt_image which, void* host, size_t bytes) try {
  if (!s) return PT_ERR_INVALID_ARG;
  JobPtr j;
  {
    std::lock_guard<std::mutex> g(s->mu);
    j = find_job(s, id);
    if (!j) {
      s->err = "unknown job id";
      return PT_ERR_INVALID_ARG;
    }
    if (j->state != ST_DONE) {
      s->err = "job is not done";
      return PT_ERR_NOT_READY;
    }
    if (which != PT_IMAGE_ACCUM && which != PT_IMAGE_ALBEDO && which != PT_IMAGE_NORMAL && which != PT_IMAGE_FINAL) {
      s->err = "jobs keep the accum, albedo, normal and final images only";
      return PT_ERR_INVALID_ARG;
    }
  }
  std::lock_guard<std::mutex> g(j->io);
  if (!j->r) return srv_fail(s, PT_ERR_STATE, "job was released");
  pt_status ps = pt_renderer_read_image(j->r, which, host, bytes);
  if (ps != PT_OK) return srv_fail(s, ps, pt_renderer_last_error(j->r));
  return PT_OK;
} catch (...) {
  return server_exception_status(s);
}

pt_status pt_server_cancel(pt_server* s, uint64_t id) try {
  if (!s) return PT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  JobPtr j = find_job(s, id);
  if (!j) {
    s->err = "unknown job id";
    return PT_ERR_INVALID_ARG;
  }
  if (j->terminal()) return PT_OK;
  j->cancel = true;
  auto it = std::find(s->queue.begin(), s->queue.end(), j);
  if (it != s->queue.end()) {
    s->queue.erase(it);
    j->in.reset();
    finish_job(s, j, ST_CANCELLED, PT_ERR_CANCELLED, "cancelled while queued");
    return PT_OK;
  }
  s->cv_admit.notify_all();
  s->cv_render.notify_all();
  return PT_OK;
} catch (...) {
  return server_exception_status(s);
}

pt_status pt_server_release(pt_server* s, uint64_t id) try {
  if (!s) return PT_ERR_INVALID_ARG;
  JobPtr j;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    j = find_job(s, id);
    if (!j) {
      s->err = "unknown job id";
      return PT_ERR_INVALID_ARG;
    }
    if (!j->terminal()) {
      j->cancel = true;
      auto it = std::find(s->queue.begin(), s->queue.end(), j);
      if (it != s->queue.end()) {
        s->queue.erase(it);
        j->in.reset();
        finish_job(s, j, ST_CANCELLED, PT_ERR_CANCELLED, "cancelled while queued");
      }
      s->cv_admit.notify_all();
      s->cv_render.notify_all();
      s->cv_done.wait(lk, [&] { return j->terminal(); });
    }
    if (j->state == ST_DONE) s->resident -= j->est;
    j->est = 0;
    s->jobs.erase(id);
    s->cv_admit.notify_all();
  }
  destroy_renderer(j);
  return PT_OK;
} catch (...) {
  return server_exception_status(s);
}

pt_status pt_server_pause(pt_server* s, int32_t paused) try {
  if (!s) return PT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  s->paused = paused != 0;
  s->cv_render.notify_all();
  return PT_OK;
} catch (...) {
  return server_exception_status(s);
}

pt_status pt_server_get_stats(pt_server* s, pt_server_stats* out) try {
  if (!s || !out) return PT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->st;
  out->jobs_queued = (uint32_t)s->queue.size() + s->admitting;
  out->jobs_running = (uint32_t)s->running.size();
  out->resident_bytes = s->resident;
  out->uptime_ms = s->now_ms();
  return PT_OK;
} catch (...) {
  return server_exception_status(s);
}

}  // extern "C"
