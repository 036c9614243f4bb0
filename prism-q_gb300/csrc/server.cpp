// Job server: continuous batching of independent MD jobs on one GPU.
//
// The reference runs one NhsAmberFusedEngine per system and has no batched or
// served form (parallel replicas bail out, fused_engine.rs:18306, :18433).
// Here one worker thread owns a batch arena sized from the caller's HBM
// budget.  Jobs are validated and lowered on the submitting thread; the worker
// admits them whenever their atom and term ranges fit in the arena's free
// space, advances all resident jobs together, and retires finished jobs at
// chunk boundaries:
//
//   loop:
//     admit queued jobs that fit (arrival order; a job that does not fit may
//       be overtaken by later ones for at most max_bypass_s, after which
//       admission waits for it)
//     chunk = min(chunk_steps, steps left of every resident job)
//     prismq_batch_step(chunk)          -- one captured graph per step
//     retire jobs that finished or whose status word is set
//
// A chunk ends exactly where the nearest job finishes, so every job runs
// exactly its n_steps, and splitting a run into chunks gives the same bits as
// one call.  Per-system trajectories do not depend on the other residents.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <list>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pq_host.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  int64_t id = 0;
  uint64_t tag = 0;
  pq::PreparedSystem* prep = nullptr;
  int32_t n_atoms = 0;
  int64_t n_steps = 0, remaining = 0;
  float* xout = nullptr;
  float* vout = nullptr;
  double t_submit = 0.0, t_start = 0.0;
  int32_t slot = -1;
  int64_t step0 = 0;  // the system's step counter at admission (a resumed job's start)
  bool has_protocol = false;
  prismq_protocol protocol{};
  std::vector<char> resume;  // checkpoint to start from (empty: the topology's own state)
  void* snap = nullptr;      // where the final checkpoint goes
  size_t snap_cap = 0;
  size_t snap_len = 0;       // bytes written there at retirement
};

void copy_message(char* dst, size_t cap, const std::string& msg) {
  const size_t n = std::min(cap - 1, msg.size());
  std::memcpy(dst, msg.data(), n);
  dst[n] = '\0';
}

}  // namespace

struct prismq_server {
  prismq_batch* batch = nullptr;
  int device = 0;
  int32_t max_systems = 1024;
  int32_t chunk_steps = 50;
  double max_bypass_s = 1.0;
  int64_t capacity_atoms = 0, device_bytes = 0;
  Clock::time_point t0;

  std::mutex mu;
  std::condition_variable cv_work;  // worker: new jobs or stop
  std::condition_variable cv_done;  // pollers: new results
  bool stop = false;
  std::list<Job> queue;     // submitted, not yet admitted (arrival order)
  std::vector<Job> resident;  // owned by the worker thread
  std::vector<prismq_job_result> results;
  int64_t next_id = 1;
  prismq_server_stats st{};
  std::thread worker;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  prismq_job_result make_result(const Job& j, prismq_status status, int64_t steps_done, const std::string& msg) {
    prismq_job_result r;
    std::memset(&r, 0, sizeof(r));
    r.job_id = j.id;
    r.tag = j.tag;
    r.status = status;
    r.n_atoms = j.n_atoms;
    r.steps_done = steps_done;
    r.submit_s = j.t_submit;
    r.start_s = j.t_start;
    r.end_s = now();
    copy_message(r.message, sizeof(r.message), msg);
    return r;
  }

  // Admit queued jobs in arrival order.  Called with `lk` held; the lock is
  // dropped around each admission (uploads) so submitters are not blocked.
  void admit(std::unique_lock<std::mutex>& lk) {
    auto it = queue.begin();
    while (it != queue.end() && (int32_t)resident.size() < max_systems) {
      Job& j = *it;
      pq::PreparedSystem* prep = j.prep;
      lk.unlock();
      int32_t slot = -1;
      prismq_status rc = pq::admit_prepared(batch, prep, &slot);
      const bool admitted = rc == PRISMQ_OK;
      if (rc == PRISMQ_OK && !j.resume.empty())
        rc = prismq_batch_checkpoint_restore(batch, slot, j.resume.data(), j.resume.size());
      int64_t step0 = 0;
      if (rc == PRISMQ_OK && !j.resume.empty()) rc = prismq_batch_get_step(batch, slot, &step0);
      if (rc == PRISMQ_OK && j.has_protocol) rc = prismq_batch_set_protocol(batch, slot, &j.protocol);
      const std::string msg = rc != PRISMQ_OK ? prismq_last_error() : "";
      if (admitted && rc != PRISMQ_OK) {
        prismq_batch_remove_system(batch, slot);
        if (rc == PRISMQ_E_CAPACITY) rc = PRISMQ_E_INVALID;  // only admission may defer a job
      }
      lk.lock();
      if (rc == PRISMQ_OK) {
        j.slot = slot;
        j.t_start = now();
        j.step0 = step0;
        pq::free_prepared(j.prep);  // uploaded; the host copy is no longer needed
        j.prep = nullptr;
        std::vector<char>().swap(j.resume);
        resident.push_back(j);
        it = queue.erase(it);
        continue;
      }
      if (rc == PRISMQ_E_CAPACITY && !resident.empty()) {
        // does not fit now; later jobs may overtake it only for a while
        const bool head = it == queue.begin();
        if (max_bypass_s <= 0.0 || (head && now() - j.t_submit > max_bypass_s)) break;
        ++it;
        continue;
      }
      results.push_back(make_result(j, rc, 0, msg));
      st.failed += 1;
      pq::free_prepared(j.prep);
      it = queue.erase(it);
      cv_done.notify_all();
    }
  }

  void run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
      admit(lk);
      if (resident.empty()) {
        // nothing on the GPU: sleep until a submit (or a bypass deadline)
        cv_work.wait_for(lk, std::chrono::milliseconds(queue.empty() ? 1000 : 5));
        continue;
      }
      int64_t chunk = chunk_steps;
      for (const Job& j : resident) chunk = std::min(chunk, j.remaining);
      lk.unlock();
      const double t_a = now();
      const prismq_status rc = prismq_batch_step(batch, chunk);
      const std::string step_msg = rc != PRISMQ_OK ? prismq_last_error() : "";
      const double t_b = now();
      // retire finished and failed jobs (outside the lock: device copies)
      std::vector<prismq_job_result> done;
      std::vector<Job> keep;
      double atom_steps = 0.0;
      int64_t completed = 0, failed = 0;
      for (Job& j : resident) {
        prismq_status js = PRISMQ_OK;
        std::string msg;
        if (rc != PRISMQ_OK) {
          js = prismq_batch_status(batch, j.slot);
          if (js != PRISMQ_OK) msg = prismq_last_error();
        }
        if (js == PRISMQ_OK) {
          j.remaining -= chunk;
          atom_steps += (double)j.n_atoms * (double)chunk;
          if (j.remaining > 0) {
            keep.push_back(j);
            continue;
          }
          js = prismq_batch_get_state(batch, j.slot, j.xout, j.vout);
          if (js != PRISMQ_OK) msg = prismq_last_error();
          if (js == PRISMQ_OK && j.snap) {
            js = prismq_batch_checkpoint_save(batch, j.slot, j.snap, j.snap_cap, &j.snap_len);
            if (js != PRISMQ_OK) msg = prismq_last_error();
          }
        }
        int64_t steps_done = j.n_steps;
        if (js != PRISMQ_OK) {
          int64_t s = 0;
          steps_done = prismq_batch_get_step(batch, j.slot, &s) == PRISMQ_OK ? s - j.step0 : j.n_steps - j.remaining;
          if (msg.empty()) msg = step_msg;
        }
        prismq_batch_remove_system(batch, j.slot);
        done.push_back(make_result(j, js, steps_done, msg));
        done.back().snapshot_len = js == PRISMQ_OK ? j.snap_len : 0;
        (js == PRISMQ_OK ? completed : failed) += 1;
      }
      lk.lock();
      resident.swap(keep);
      st.chunks += 1;
      st.busy_s += t_b - t_a;
      st.atom_steps += atom_steps;
      st.completed += completed;
      st.failed += failed;
      if (!done.empty()) {
        results.insert(results.end(), done.begin(), done.end());
        cv_done.notify_all();
      }
    }
  }
};

extern "C" {

void prismq_server_config_default(prismq_server_config* cfg) {
  if (!cfg) return;
  cfg->max_systems = 1024;
  cfg->chunk_steps = 50;
  cfg->max_bypass_s = 1.0;
}

prismq_status prismq_server_create(int64_t max_hbm_bytes, const prismq_server_config* cfg, prismq_server** out) {
  if (!out) {
    pq::set_last_error("out is NULL");
    return PRISMQ_E_INVALID;
  }
  *out = nullptr;
  prismq_server_config c;
  prismq_server_config_default(&c);
  if (cfg) {
    if (cfg->max_systems > 0) c.max_systems = cfg->max_systems;
    if (cfg->chunk_steps > 0) c.chunk_steps = cfg->chunk_steps;
    if (cfg->max_bypass_s >= 0.0) c.max_bypass_s = cfg->max_bypass_s;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    pq::set_last_error("no CUDA device visible");
    return PRISMQ_E_NO_DEVICE;
  }
  auto* S = new prismq_server();
  S->max_systems = c.max_systems;
  S->chunk_steps = c.chunk_steps;
  S->max_bypass_s = c.max_bypass_s;
  cudaGetDevice(&S->device);
  const prismq_status rc =
      pq::batch_create_for_bytes(max_hbm_bytes, c.max_systems, &S->batch, &S->capacity_atoms, &S->device_bytes);
  if (rc != PRISMQ_OK) {
    delete S;
    return rc;
  }
  S->t0 = Clock::now();
  S->worker = std::thread([S] { S->run(); });
  *out = S;
  return PRISMQ_OK;
}

prismq_status prismq_server_submit(prismq_server* s, const prismq_job* job, int64_t* job_id) {
  if (!s || !job || !job_id) {
    pq::set_last_error("NULL argument");
    return PRISMQ_E_INVALID;
  }
  if (job->n_steps < 1) {
    pq::set_last_error("n_steps must be >= 1");
    return PRISMQ_E_INVALID;
  }
  if (job->params.precision != PRISMQ_PRECISION_FP32) {
    pq::set_last_error("the server runs FP32 (production) jobs");
    return PRISMQ_E_INVALID;
  }
  if (job->protocol) {  // validated here so a bad protocol fails the submit, not the job
    float probe[3];
    const prismq_status prc = prismq_protocol_eval(job->protocol, 1, probe);
    if (prc != PRISMQ_OK) return prc;
  }
  pq::PreparedSystem* prep = nullptr;
  const prismq_status rc = pq::prepare_system(job->topology, &job->params, &prep);
  if (rc != PRISMQ_OK) return rc;
  const int32_t n = pq::prepared_atoms(prep);
  if ((int64_t)n > s->capacity_atoms) {
    pq::free_prepared(prep);
    pq::set_last_error("job has " + std::to_string(n) + " atoms; the server arena holds " +
                       std::to_string(s->capacity_atoms));
    return PRISMQ_E_CAPACITY;
  }
  size_t ckpt = 0;
  prismq_checkpoint_size_for_atoms(n, &ckpt);
  if ((job->snapshot_out && job->snapshot_cap < ckpt) || (job->resume && job->resume_len != ckpt)) {
    pq::free_prepared(prep);  // the blob's own checks run at admission; its size is known now
    pq::set_last_error("snapshot buffer or resume blob is not " + std::to_string(ckpt) + " bytes");
    return PRISMQ_E_INVALID;
  }
  Job j;
  j.tag = job->tag;
  j.prep = prep;
  j.n_atoms = n;
  j.n_steps = j.remaining = job->n_steps;
  j.xout = job->positions_out;
  j.vout = job->velocities_out;
  if (job->protocol) {
    j.has_protocol = true;
    j.protocol = *job->protocol;
  }
  if (job->resume && job->resume_len > 0) {
    const char* r = static_cast<const char*>(job->resume);
    j.resume.assign(r, r + job->resume_len);
  }
  j.snap = job->snapshot_out;
  j.snap_cap = job->snapshot_out ? job->snapshot_cap : 0;
  {
    std::lock_guard<std::mutex> g(s->mu);
    j.id = s->next_id++;
    j.t_submit = s->now();
    s->queue.push_back(j);
    s->st.submitted += 1;
  }
  s->cv_work.notify_one();
  *job_id = j.id;
  return PRISMQ_OK;
}

prismq_status prismq_server_poll(prismq_server* s, prismq_job_result* out, int32_t cap, int32_t* n,
                                 int32_t wait_ms) {
  if (!s || !n || (cap > 0 && !out) || cap < 0) {
    pq::set_last_error("invalid poll arguments");
    return PRISMQ_E_INVALID;
  }
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->results.empty() && wait_ms > 0)
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [s] { return !s->results.empty(); });
  const int32_t k = std::min<int32_t>(cap, (int32_t)s->results.size());
  for (int32_t i = 0; i < k; ++i) out[i] = s->results[i];
  s->results.erase(s->results.begin(), s->results.begin() + k);
  *n = k;
  return PRISMQ_OK;
}

prismq_status prismq_server_stats_get(prismq_server* s, prismq_server_stats* out) {
  if (!s || !out) {
    pq::set_last_error("NULL argument");
    return PRISMQ_E_INVALID;
  }
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->st;
  out->queued = (int64_t)s->queue.size();
  out->resident_jobs = (int64_t)s->resident.size();
  int64_t atoms = 0;
  for (const Job& j : s->resident) atoms += j.n_atoms;
  out->resident_atoms = atoms;
  out->capacity_atoms = s->capacity_atoms;
  out->device_bytes = s->device_bytes;
  out->uptime_s = s->now();
  return PRISMQ_OK;
}

void prismq_server_destroy(prismq_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (Job& j : s->queue) pq::free_prepared(j.prep);
  prismq_batch_destroy(s->batch);
  delete s;
}

}  // extern "C"
