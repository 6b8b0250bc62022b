// Serving loop: transform jobs of mixed sizes, kinds and precisions admitted under an HBM
// budget as they arrive, with continuous batching over concurrent streams (no counterpart in
// the reference, whose API runs one transform per call, build/exec.C:101-223).
//
// A job is (forward 3D plan, backward 3D plan, derivative direction, input, output): the input
// field is copied into HBM, transformed forward with the i*k derivative fused into the stage of
// dim idir, transformed back, and the result copied out.  Inputs and outputs may be host memory
// (copied on the job's stream, overlapping other jobs' kernels) or device memory.
//
// One dispatcher thread owns the device work:
//   - jobs submitted with an arrival time wait in a time-ordered list until that time (trace
//     replay), then join the admission queue
//   - a job is admitted when a slot (stream) is free and its HBM need (input/output field,
//     spectrum, two scratch fields) fits in what the budget has left; the queue is scanned in
//     arrival order with a bounded look-ahead, and the head job may not be passed over for
//     longer than a set time, so large jobs are not starved
//   - an admitted job allocates its fields from a stream-ordered memory pool (cudaMallocAsync;
//     the pool keeps freed blocks cached, so steady state makes no driver allocation), queues
//     its copies and stage kernels on its slot's stream, and ends with a host callback that
//     stamps the completion time and wakes the dispatcher
//   - a completed job returns its memory to the pool (cudaFreeAsync) and its slot
// Plans, twiddle tables and kernel modules stay resident across jobs; every running job's
// kernels overlap on the device with the other slots' work.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "kernels.h"
#include "p3dfft_gb300.h"
#include "runtime.h"

namespace p3d {

enum JobState { J_PENDING = 0, J_QUEUED, J_RUNNING, J_DONE, J_FAILED };

struct Server;

struct SJob {
  Server *srv = nullptr;
  int id = 0;
  int plan_f = -1, plan_b = -1, idir = -1;
  const void *in = nullptr;
  void *out = nullptr;
  size_t in_bytes = 0, spec_bytes = 0, scratch_bytes = 0, need = 0;
  double t_arrival = 0, t_admit = 0, t_done = 0;
  std::atomic<int> state{J_PENDING};
  bool finished = false;  // set by the completion callback
  int slot = -1;
  void *d_in = nullptr, *d_spec = nullptr, *d_s0 = nullptr, *d_s1 = nullptr;
  void *set = nullptr;
  int err = E_OK;
  bool inject_alloc_failure = false;  // test hook: its device allocation fails at launch
};

struct Server {
  int device = 0;
  size_t budget = 0, in_use = 0, peak = 0;
  int nslots = 8;
  double max_bypass_s = 0.05;  // longest time the head job may be passed over
  int lookahead = 64;
  std::vector<cudaStream_t> streams;
  std::vector<SJob *> slot_job;
  cudaMemPool_t pool = nullptr;
  std::chrono::steady_clock::time_point t0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  std::condition_variable cv_done;
  std::multimap<double, SJob *> future;  // submitted, arrival time not reached
  std::deque<SJob *> queue;              // arrived, waiting for admission
  std::vector<SJob *> jobs;              // all jobs by id
  std::atomic<int> callbacks{0};         // completions not yet retired
  long long completed = 0, failed = 0, admitted = 0;
  double host_launch_s = 0, host_release_s = 0;  // dispatcher time spent queueing / releasing jobs
  int max_running = 0;
  bool admit_dirty = false;  // queue, slots or budget changed since the last admission pass
  bool stop = false;

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

static std::mutex g_smu;
static std::vector<Server *> g_servers;

static Server *get_server(int h) {
  std::lock_guard<std::mutex> g(g_smu);
  if (h < 0 || h >= (int)g_servers.size()) return nullptr;
  return g_servers[h];
}

// runs on a CUDA callback thread: no CUDA calls here
static void CUDART_CB job_done_cb(void *arg) {
  SJob *j = static_cast<SJob *>(arg);
  Server *S = j->srv;
  {
    std::lock_guard<std::mutex> g(S->mu);
    j->t_done = S->now();
    j->finished = true;
    S->callbacks++;
  }
  S->cv.notify_all();
}

// Returns the job's fields to the pool, ordered after its work on stream `st`.  CUDA calls only:
// the caller does not hold the server lock (a host callback may be waiting for it).
static void release_job_memory(SJob *j, cudaStream_t st) {
  for (void **p : {&j->d_in, &j->d_spec, &j->d_s0, &j->d_s1}) {
    if (*p) cudaFreeAsync(*p, st);
    *p = nullptr;
  }
  if (j->set) scratch_set_destroy(j->set);
  j->set = nullptr;
}

// Queues the job's work on its slot stream; returns E_OK or an error (the job is then failed).
// Called without the server lock.
static int launch_job(Server *S, SJob *j) {
  cudaStream_t st = S->streams[j->slot];
  auto alloc = [&](void **p, size_t b) {
    return cudaMallocFromPoolAsync(p, std::max<size_t>(b, 256), S->pool, st) == cudaSuccess;
  };
  if (j->inject_alloc_failure || !alloc(&j->d_in, j->in_bytes) || !alloc(&j->d_spec, j->spec_bytes) ||
      !alloc(&j->d_s0, j->scratch_bytes) || !alloc(&j->d_s1, j->scratch_bytes)) {
    cudaGetLastError();
    return E_CUDA;
  }
  j->set = scratch_set_wrap(j->d_s0, j->d_s1, std::max<size_t>(j->scratch_bytes, 256));
  if (cudaMemcpyAsync(j->d_in, j->in, j->in_bytes, cudaMemcpyDefault, st) != cudaSuccess) return E_CUDA;
  int rc = exec_plan_on(j->plan_f, j->d_in, j->d_spec, j->idir, st, j->set, false);
  if (rc != E_OK) return rc;
  rc = exec_plan_on(j->plan_b, j->d_spec, j->d_in, -1, st, j->set, false);  // result over the input field
  if (rc != E_OK) return rc;
  if (cudaMemcpyAsync(j->out, j->d_in, j->in_bytes, cudaMemcpyDefault, st) != cudaSuccess) return E_CUDA;
  if (cudaLaunchHostFunc(st, job_done_cb, j) != cudaSuccess) return E_CUDA;
  return E_OK;
}

// Admission pass (server lock held): fills free slots from the queue.
static void admit(Server *S, double t, std::vector<SJob *> &start) {
  for (;;) {
    if (S->queue.empty()) return;
    int slot = -1;
    for (int s = 0; s < S->nslots; s++)
      if (!S->slot_job[s]) {
        slot = s;
        break;
      }
    if (slot < 0) return;
    const bool head_starving = t - S->queue.front()->t_arrival > S->max_bypass_s;
    const int scan = head_starving ? 1 : std::min<int>(S->lookahead, (int)S->queue.size());
    SJob *pick = nullptr;
    for (int q = 0; q < scan; q++) {
      SJob *j = S->queue[q];
      if (j->need > S->budget) {  // can never fit
        j->err = E_TOO_LARGE;
        j->state = J_FAILED;
        S->failed++;
        S->queue.erase(S->queue.begin() + q);
        S->cv_done.notify_all();
        pick = j;
        break;
      }
      if (S->in_use + j->need > S->budget) continue;
      S->queue.erase(S->queue.begin() + q);
      j->slot = slot;
      j->t_admit = t;
      j->state = J_RUNNING;
      S->slot_job[slot] = j;
      S->in_use += j->need;
      S->peak = std::max(S->peak, S->in_use);
      S->admitted++;
      int running = 0;
      for (auto *r : S->slot_job) running += r != nullptr;
      S->max_running = std::max(S->max_running, running);
      start.push_back(j);
      pick = j;
      break;
    }
    if (!pick) return;  // nothing in reach fits now
  }
}

// Dispatcher: under the lock it collects completions, releases arrivals and picks admissions;
// the CUDA work (freeing and launching) is done with the lock released, so the completion
// callbacks, which take the lock, never wait on a thread that waits on the GPU.
static void dispatcher(Server *S) {
  cudaSetDevice(S->device);
  std::vector<SJob *> done, start;
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    done.clear();
    start.clear();
    if (S->callbacks > 0) {
      for (int s = 0; s < S->nslots; s++) {
        SJob *j = S->slot_job[s];
        if (j && j->finished && j->state == J_RUNNING) {
          done.push_back(j);
          S->slot_job[s] = nullptr;  // its stream runs the frees before any new job's work
          S->callbacks--;
        }
      }
    }
    const double t = S->now();
    while (!S->future.empty() && S->future.begin()->first <= t) {
      SJob *j = S->future.begin()->second;
      S->future.erase(S->future.begin());
      j->state = J_QUEUED;
      S->queue.push_back(j);
      S->admit_dirty = true;
    }
    if (S->admit_dirty || !done.empty()) {
      S->admit_dirty = false;
      admit(S, t, start);
    }
    if (done.empty() && start.empty()) {
      bool busy = false;
      for (auto *r : S->slot_job) busy |= r != nullptr;
      if (S->stop && !busy && S->queue.empty() && S->future.empty()) break;
      auto ready = [&] {
        return S->callbacks > 0 || S->admit_dirty || S->stop ||
               (!S->future.empty() && S->future.begin()->first <= S->now());
      };
      double dt = 0.05;
      if (!S->future.empty()) dt = std::min(dt, std::max(0.0, S->future.begin()->first - S->now()));
      S->cv.wait_for(lk, std::chrono::duration<double>(dt), ready);
      continue;
    }
    lk.unlock();
    const double h0 = S->now();
    for (SJob *j : done) release_job_memory(j, S->streams[j->slot]);
    const double h1 = S->now();
    std::vector<std::pair<SJob *, int>> failed;
    for (SJob *j : start) {
      const int rc = launch_job(S, j);
      if (rc != E_OK) {
        cudaStreamSynchronize(S->streams[j->slot]);
        release_job_memory(j, S->streams[j->slot]);
        failed.push_back({j, rc});
      }
    }
    const double h2 = S->now();
    lk.lock();
    S->host_release_s += h1 - h0;
    S->host_launch_s += h2 - h1;
    for (SJob *j : done) {
      S->in_use -= j->need;
      j->state = J_DONE;
      S->completed++;
    }
    for (auto &f : failed) {
      SJob *j = f.first;
      S->in_use -= j->need;
      j->err = f.second;
      j->state = J_FAILED;
      S->slot_job[j->slot] = nullptr;
      S->failed++;
    }
    if (!done.empty() || !failed.empty()) S->admit_dirty = true;
    S->cv_done.notify_all();
  }
}

}  // namespace p3d

using namespace p3d;

extern "C" {

int p3dfft_gb300_server_create(long long hbm_budget_bytes, int nslots) {
  if (hbm_budget_bytes <= 0 || nslots < 1 || nslots > 256) {
    record_error(E_BAD_ARG, "server: budget must be > 0 and slots 1..256");
    return -1;
  }
  if (!device_ready()) return -1;
  if (p3dfft_gb300_preload_kernels() != E_OK) return -1;
  Server *S = new Server();
  cudaGetDevice(&S->device);
  S->budget = (size_t)hbm_budget_bytes;
  S->nslots = nslots;
  S->streams.resize(nslots);
  S->slot_job.assign(nslots, nullptr);
  for (auto &s : S->streams) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = S->device;
  if (cudaMemPoolCreate(&S->pool, &props) != cudaSuccess) {
    cudaGetLastError();
    for (auto s : S->streams) cudaStreamDestroy(s);
    delete S;
    record_error(E_CUDA, "server: memory pool creation failed");
    return -1;
  }
  unsigned long long thr = (unsigned long long)hbm_budget_bytes;  // keep freed blocks cached
  cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &thr);
  S->t0 = std::chrono::steady_clock::now();
  S->th = std::thread(dispatcher, S);
  std::lock_guard<std::mutex> g(g_smu);
  g_servers.push_back(S);
  return (int)g_servers.size() - 1;
}

double p3dfft_gb300_server_clock(int srv) {
  Server *S = get_server(srv);
  return S ? S->now() : -1.0;
}

int p3dfft_gb300_server_submit(int srv, int plan_fwd, int plan_bwd, int idir, const void *in, void *out,
                               double arrival_s) {
  Server *S = get_server(srv);
  if (!S) {
    record_error(E_BAD_ARG, "server: invalid handle");
    return -1;
  }
  size_t fi = 0, fo = 0, fs = 0, bi = 0, bo = 0, bs = 0;
  int fp = 0, bp = 0;
  if (plan3d_sizes(plan_fwd, &fi, &fo, &fs, &fp) != E_OK || plan3d_sizes(plan_bwd, &bi, &bo, &bs, &bp) != E_OK)
    return -1;
  if (fo != bi || bo != fi || fp != bp) {
    record_error(E_BAD_ARG, "server: backward plan does not invert the forward plan's field sizes");
    return -1;
  }
  if (!in || !out || idir > 2) {
    record_error(E_BAD_ARG, "server: null data pointer or derivative direction out of range");
    return -1;
  }
  SJob *j = new SJob();
  j->srv = S;
  j->plan_f = plan_fwd;
  j->plan_b = plan_bwd;
  j->idir = idir;
  j->in = in;
  j->out = out;
  j->in_bytes = fi;
  j->spec_bytes = fo;
  j->scratch_bytes = std::max(fs, bs);
  auto round = [](size_t b) { return (std::max<size_t>(b, 256) + 255) & ~(size_t)255; };
  j->need = round(fi) + round(fo) + 2 * round(j->scratch_bytes);
  {
    std::lock_guard<std::mutex> g(S->mu);
    j->id = (int)S->jobs.size();
    S->jobs.push_back(j);
    const double t = S->now();
    j->t_arrival = arrival_s < 0 ? t : arrival_s;
    if (j->t_arrival <= t) {
      j->state = J_QUEUED;
      S->queue.push_back(j);
      S->admit_dirty = true;
    } else {
      S->future.emplace(j->t_arrival, j);
    }
  }
  S->cv.notify_all();
  return j->id;
}

int p3dfft_gb300_server_inject_alloc_failure(int srv, int job) {
  Server *S = get_server(srv);
  if (!S) {
    record_error(E_BAD_ARG, "server: invalid handle");
    return E_BAD_ARG;
  }
  std::lock_guard<std::mutex> g(S->mu);
  if (job < 0 || job >= (int)S->jobs.size() || S->jobs[job]->state == J_RUNNING || S->jobs[job]->state == J_DONE ||
      S->jobs[job]->state == J_FAILED) {
    record_error(E_BAD_ARG, "server: the job is not waiting for admission");
    return E_BAD_ARG;
  }
  S->jobs[job]->inject_alloc_failure = true;
  return E_OK;
}

// 0 done, 1 not yet (timeout), negative: the job failed with that error code negated
int p3dfft_gb300_server_wait(int srv, int job, double timeout_s) {
  Server *S = get_server(srv);
  if (!S || job < 0) return -E_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  if (job >= (int)S->jobs.size()) return -E_BAD_ARG;
  SJob *j = S->jobs[job];
  auto fin = [&] { return j->state == J_DONE || j->state == J_FAILED; };
  if (timeout_s < 0) S->cv_done.wait(lk, fin);
  else S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), fin);
  if (j->state == J_DONE) return 0;
  if (j->state == J_FAILED) return -j->err;
  return 1;
}

int p3dfft_gb300_server_drain(int srv) {
  Server *S = get_server(srv);
  if (!S) return E_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  S->cv_done.wait(lk, [&] { return S->completed + S->failed == (long long)S->jobs.size(); });
  return S->failed ? E_PLAN : E_OK;
}

// t[0] arrival, t[1] admission, t[2] completion (seconds on the server clock)
int p3dfft_gb300_server_job_times(int srv, int job, double *t) {
  Server *S = get_server(srv);
  if (!S || !t) return E_BAD_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  if (job < 0 || job >= (int)S->jobs.size()) return E_BAD_ARG;
  SJob *j = S->jobs[job];
  t[0] = j->t_arrival;
  t[1] = j->t_admit;
  t[2] = j->t_done;
  return j->state == J_DONE ? E_OK : (j->state == J_FAILED ? -j->err : E_PLAN);
}

// stats: completed, failed, admitted, peak HBM bytes in use, budget bytes, most jobs running at
// once, dispatcher seconds spent queueing jobs' work, and releasing their memory
int p3dfft_gb300_server_stats(int srv, double *stats, int n) {
  Server *S = get_server(srv);
  if (!S || !stats) return E_BAD_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  const double v[8] = {(double)S->completed, (double)S->failed, (double)S->admitted, (double)S->peak,
                       (double)S->budget, (double)S->max_running, S->host_launch_s, S->host_release_s};
  for (int i = 0; i < n && i < 8; i++) stats[i] = v[i];
  return E_OK;
}

int p3dfft_gb300_server_destroy(int srv) {
  Server *S;
  {
    std::lock_guard<std::mutex> g(g_smu);
    if (srv < 0 || srv >= (int)g_servers.size() || !g_servers[srv]) return E_BAD_ARG;
    S = g_servers[srv];
    g_servers[srv] = nullptr;
  }
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  S->th.join();
  for (auto s : S->streams) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  cudaMemPoolDestroy(S->pool);
  for (auto *j : S->jobs) delete j;
  delete S;
  return E_OK;
}

}  // extern "C"
