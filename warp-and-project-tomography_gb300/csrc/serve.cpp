// Request loop for many reconstructions on one GPU (include/wap/wap_serve.h).
//
// Jobs wait in a FIFO queue until their device footprint
// (wap_job_device_bytes) fits in what the budget has left; admission is
// first-fit over the queue, so a large job at the head does not hold back
// small ones behind it, except that a job waiting longer than kHeadPatience
// seconds blocks later admissions until it fits (no starvation).  Worker
// threads take the admitted job that has run the fewest steps and is not
// being stepped, run its next outer-iteration step on its own context and
// stream, and put it back; so up to `workers` jobs run concurrently on the
// GPU and every admitted job keeps moving.  A job's steps run strictly in
// order on its own context, so its result is the same alone or in the mix.
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

#include <cuda_runtime.h>

#include "wap/wap.h"
#include "wap/wap_serve.h"
#include "wap_internal.h"
#include "c_boundary.h"

namespace {

constexpr double kHeadPatience = 2.0;

struct Job {
  long long id = 0;
  wap_job_desc desc{};
  std::vector<double> angles;
  std::vector<float> projs;
  wap_job_info info{};
  wap_ctx *ctx = nullptr;
  int nsteps = 0;       // steps per outer iteration
  long long total = 0;  // steps of the whole job
  bool busy = false;
  std::vector<std::vector<float>> result;
};

}  // namespace

struct wap_server {
  int device = 0;
  size_t budget = 0;
  std::chrono::steady_clock::time_point t0;
  std::mutex m;
  std::condition_variable cv;       // work available / state change
  std::condition_variable done_cv;  // a job finished
  std::deque<Job *> queue;
  std::vector<Job *> active;
  std::map<long long, std::unique_ptr<Job>> jobs;
  size_t in_use = 0, peak = 0;
  long long next_id = 1;
  bool stop = false;
  std::vector<std::thread> workers;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  // Admission under the lock: first-fit over the queue, with the head's
  // patience rule.
  void admit_locked(std::vector<Job *> &admitted) {
    admitted.reserve(queue.size());  // may throw; nothing has changed yet
    const double t = now();
    for (auto it = queue.begin(); it != queue.end();) {
      Job *j = *it;
      if (in_use + j->info.device_bytes <= budget) {
        in_use += j->info.device_bytes;
        peak = std::max(peak, in_use);
        j->info.state = WAP_JOB_RUNNING;
        j->info.t_admit = t;
        j->busy = true;  // the admitting worker sets it up
        admitted.push_back(j);
        it = queue.erase(it);
        continue;
      }
      if (it == queue.begin() && t - j->info.t_submit > kHeadPatience) break;
      ++it;
    }
  }

  void finish_locked(Job *j, int status) {
    j->info.state = status == WAP_OK ? WAP_JOB_DONE : WAP_JOB_FAILED;
    j->info.status = status;
    j->info.t_done = now();
    in_use -= j->info.device_bytes;
    active.erase(std::remove(active.begin(), active.end(), j), active.end());
    j->busy = false;
    done_cv.notify_all();
    cv.notify_all();
  }

  // Context, projections and level state of a newly admitted job.
  int setup(Job *j) {
    int r = wap_create(&j->ctx, &j->desc.scan, j->angles.data(), device);
    if (r != WAP_OK) return r;
    if (j->desc.flow_bits == 16 && (r = wap_set_tuning(j->ctx, "flow_bits", 16)) != WAP_OK) return r;
    if ((r = wap_upload_projections(j->ctx, j->projs.data())) != WAP_OK) return r;
    if ((r = wap_level_setup(j->ctx, 0)) != WAP_OK) return r;
    j->nsteps = wap_outer_iteration_nsteps(j->ctx, &j->desc.sched);
    if (j->nsteps <= 0) return WAP_EINVAL;
    j->total = (long long)j->nsteps * std::max(j->desc.outer_iterations, 0);
    std::vector<float>().swap(j->projs);  // the device copy is the job's state now
    return WAP_OK;
  }

  int collect(Job *j) {
    const int F = wap_level_nframes(j->ctx);
    const size_t nv = (size_t)j->desc.scan.vol[0] * j->desc.scan.vol[1] * j->desc.scan.vol[2];
    j->result.assign(F, std::vector<float>(nv));
    for (int f = 0; f < F; ++f) {
      const int r = wap_frame_volume_download(j->ctx, f, j->result[f].data());
      if (r != WAP_OK) return r;
    }
    return WAP_OK;
  }

  void release_ctx(Job *j) {
    if (j->ctx) wap_destroy(j->ctx);
    j->ctx = nullptr;
  }

  // A worker's call into the library or its own host allocations: an
  // exception (host memory) becomes the job's failure status, so it never
  // leaves the worker thread.
  template <class Fn>
  static int guarded(Fn &&fn) {
    try {
      return fn();
    } catch (const std::bad_alloc &) {
      return WAP_ENOMEM;
    } catch (...) {
      return WAP_EHOST;
    }
  }

  // Stops and joins the workers (destruction, or a failed start).
  void stop_workers() {
    {
      std::lock_guard<std::mutex> lk(m);
      stop = true;
    }
    cv.notify_all();
    for (auto &t : workers) t.join();
    workers.clear();
  }

  void worker() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(m);
    while (!stop) {
      std::vector<Job *> admitted;
      try {
        admit_locked(admitted);
      } catch (const std::bad_alloc &) {  // no host memory for the list: admit nothing this round
        admitted.clear();
      }
      if (!admitted.empty()) {
        lk.unlock();
        for (Job *j : admitted) {
          const int r = guarded([&] { return setup(j); });
          lk.lock();
          if (r != WAP_OK) {
            release_ctx(j);
            finish_locked(j, r);
          } else {
            j->busy = false;
            active.push_back(j);
            cv.notify_all();
          }
          lk.unlock();
        }
        lk.lock();
        continue;
      }
      Job *pick = nullptr;
      for (Job *j : active)
        if (!j->busy && (!pick || j->info.steps < pick->info.steps)) pick = j;
      if (!pick) {
        cv.wait(lk);
        continue;
      }
      pick->busy = true;
      const long long k = pick->info.steps;
      lk.unlock();
      int r = WAP_OK;
      bool last = k >= pick->total;
      if (!last) {
        r = wap_outer_iteration_step(pick->ctx, &pick->desc.sched, (int)(k % pick->nsteps), nullptr);
        last = (k + 1 >= pick->total);
      }
      if (r == WAP_OK && last) r = guarded([&] { return collect(pick); });
      if (last || r != WAP_OK) release_ctx(pick);
      lk.lock();
      if (r == WAP_OK) pick->info.steps = k + (k < pick->total ? 1 : 0);
      if (r != WAP_OK || last) finish_locked(pick, r);
      else {
        pick->busy = false;
        cv.notify_all();
      }
    }
  }
};

extern "C" {

int wap_server_create(wap_server **out, int device, size_t hbm_budget_bytes, int workers) try {
  if (!out || workers < 1 || workers > 64 || hbm_budget_bytes == 0) return WAP_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return WAP_ENODEV;
  std::unique_ptr<wap_server> s(new wap_server);
  s->device = device;
  s->budget = hbm_budget_bytes;
  s->t0 = std::chrono::steady_clock::now();
  try {
    for (int w = 0; w < workers; ++w) s->workers.emplace_back([p = s.get()] { p->worker(); });
  } catch (...) {
    s->stop_workers();  // the ones that did start, before the server goes away
    throw;
  }
  *out = s.release();
  return WAP_OK;
} WAP_CATCH

void wap_server_destroy(wap_server *s) {
  if (!s) return;
  s->stop_workers();
  for (auto &kv : s->jobs) s->release_ctx(kv.second.get());
  wap_trim_cache(s->device);  // the jobs' recycled device blocks
  delete s;
}

int wap_server_submit(wap_server *s, const wap_job_desc *job, long long *h_id) try {
  if (!s || !job || !h_id || !job->h_angles || !job->h_projs || job->outer_iterations < 1) return WAP_EINVAL;
  if (job->flow_bits != 0 && job->flow_bits != 32 && job->flow_bits != 16) return WAP_EINVAL;
  const wap_scan_desc &sc = job->scan;
  if (sc.nproj < 1 || sc.det[0] < 5 || sc.det[1] < 5) return WAP_EINVAL;
  std::unique_ptr<Job> j(new Job);
  j->desc = *job;
  j->angles.assign(job->h_angles, job->h_angles + sc.nproj);
  j->projs.assign(job->h_projs, job->h_projs + (size_t)sc.det[0] * sc.det[1] * sc.nproj);
  j->desc.h_angles = nullptr;
  j->desc.h_projs = nullptr;
  j->info.device_bytes = wap_job_device_bytes(&sc, &job->sched);
  if (j->info.device_bytes == 0) return WAP_EINVAL;
  if (job->flow_bits == 16)
    j->info.device_bytes += wap::flow_pairs_bytes(sc.vol, job->sched.flow_scales, job->sched.flow_eta);
  if (j->info.device_bytes > s->budget) return WAP_ETOOBIG;
  std::lock_guard<std::mutex> lk(s->m);
  // room for every job in the active list, so that a worker's push never
  // allocates (a failure here leaves the server unchanged)
  s->active.reserve(s->jobs.size() + 1);
  j->id = s->next_id++;
  j->info.state = WAP_JOB_QUEUED;
  j->info.status = WAP_OK;
  j->info.t_submit = s->now();
  Job *jp = j.get();
  // the map takes ownership first; if the queue cannot take the job too, the
  // map lets it go again, so a failed submit leaves no trace
  auto ins = s->jobs.emplace(jp->id, std::move(j));
  try {
    s->queue.push_back(jp);
  } catch (...) {
    s->jobs.erase(ins.first);
    throw;
  }
  *h_id = jp->id;
  s->cv.notify_all();
  return WAP_OK;
} WAP_CATCH

int wap_server_info(wap_server *s, long long id, wap_job_info *out) try {
  if (!s || !out) return WAP_EINVAL;
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return WAP_EINVAL;
  *out = it->second->info;
  return WAP_OK;
} WAP_CATCH

int wap_server_wait(wap_server *s, long long id, double timeout_s) try {
  if (!s) return WAP_EINVAL;
  std::unique_lock<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return WAP_EINVAL;
  Job *j = it->second.get();
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
  while (j->info.state == WAP_JOB_QUEUED || j->info.state == WAP_JOB_RUNNING)
    if (s->done_cv.wait_until(lk, deadline) == std::cv_status::timeout &&
        (j->info.state == WAP_JOB_QUEUED || j->info.state == WAP_JOB_RUNNING))
      return WAP_ESTATE;
  return j->info.state == WAP_JOB_DONE ? WAP_OK : j->info.status;
} WAP_CATCH

int wap_server_result(wap_server *s, long long id, int frame, float *h_vol) try {
  if (!s || !h_vol) return WAP_EINVAL;
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end() || it->second->info.state != WAP_JOB_DONE) return WAP_ESTATE;
  Job *j = it->second.get();
  if (frame < 0 || frame >= (int)j->result.size()) return WAP_EINVAL;
  std::memcpy(h_vol, j->result[frame].data(), sizeof(float) * j->result[frame].size());
  return WAP_OK;
} WAP_CATCH

int wap_server_release(wap_server *s, long long id) try {
  if (!s) return WAP_EINVAL;
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return WAP_EINVAL;
  const int st = it->second->info.state;
  if (st != WAP_JOB_DONE && st != WAP_JOB_FAILED) return WAP_ESTATE;
  s->jobs.erase(it);
  return WAP_OK;
} WAP_CATCH

double wap_server_now(const wap_server *s) { return s ? s->now() : 0.0; }

int wap_server_memory(const wap_server *s, size_t *h_in_use, size_t *h_peak) try {
  if (!s) return WAP_EINVAL;
  std::lock_guard<std::mutex> lk(const_cast<wap_server *>(s)->m);
  if (h_in_use) *h_in_use = s->in_use;
  if (h_peak) *h_peak = s->peak;
  return WAP_OK;
} WAP_CATCH

}  // extern "C"
