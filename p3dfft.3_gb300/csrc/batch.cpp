// Batched execution of many independent 3D transforms (no counterpart in the reference, whose
// transform3D::exec runs one transform per call, build/exec.C:101-223).
//
// A batch is a set of jobs; a job is an ordered list of (plan, in, out, idir) steps on device
// memory, e.g. an R2C forward followed by the C2R backward.  Two ways to run them:
//   - grouped (default): jobs with the same steps form a cohort, and each stage of a cohort runs
//     as ONE launch of its specialised kernel over the tiles of all the cohort's jobs, so the
//     batch is a few large launches instead of many small ones; cohorts run concurrently on the
//     branch streams.  Each job has its own scratch set.
//   - branches: jobs are spread over branch streams by a longest-processing-time-first
//     assignment on their HBM bytes; each branch owns one scratch set, sized for the largest plan
//     it runs, and runs its jobs one after another.
// The first exec runs the jobs eagerly (this resolves twiddle tables and scratch), then records
// the whole structure into one CUDA graph; every later exec is a single cudaGraphLaunch on the
// library stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "kernels.h"
#include "p3dfft_gb300.h"
#include "runtime.h"

namespace p3d {

struct BatchStep {
  int plan;
  const void *in;
  void *out;
  int idir;
};

struct Batch {
  int nbr = 8;
  std::map<int, std::vector<BatchStep>> jobs;
  std::vector<std::vector<int>> assign;  // branch -> job ids
  std::vector<cudaStream_t> br;
  std::vector<void *> sets;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  cudaStream_t origin = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool use_graph = true;
  bool grouped = true;          // level-synchronous grouped launches (else one stream per branch)
  bool work_list = false;       // grouped mode over all jobs: one work-list launch per kernel per level
  std::vector<void *> job_sets;          // grouped mode: one scratch set per job
  std::vector<LaunchSet *> lsets;         // grouped mode: one launch set per cohort
  std::vector<std::vector<int>> cassign;  // grouped mode: branch -> cohorts
  // work-list mode: the job at each position of each level, and one event per launch
  std::vector<std::vector<int>> level_jobs;
  std::vector<cudaEvent_t> item_ev;
  int ngroups = 0;
  bool dirty = true;
  int arith = -1;
  long long kernels = 0;  // kernels one exec launches
  double bytes = 0;       // field bytes one exec reads and writes (inputs + outputs of every step)

  ~Batch() {
    if (gexec) cudaGraphExecDestroy(gexec);
    for (auto l : lsets) launch_set_destroy(l);
    for (auto p : job_sets) scratch_set_destroy(p);
    for (auto s : br) cudaStreamDestroy(s);
    for (auto e : join) cudaEventDestroy(e);
    for (auto e : item_ev) cudaEventDestroy(e);
    for (auto p : sets) scratch_set_destroy(p);
    if (fork) cudaEventDestroy(fork);
    if (origin) cudaStreamDestroy(origin);
  }
};

static std::mutex g_bmu;
static std::vector<Batch *> g_batches;

static Batch *get_batch(int h) {
  std::lock_guard<std::mutex> g(g_bmu);
  if (h < 0 || h >= (int)g_batches.size()) return nullptr;
  return g_batches[h];
}

static int fail(int code, const char *msg) {
  record_error(code, msg);
  return code;
}

// Longest-processing-time-first assignment of jobs to branches, then one scratch set per branch.
static int prepare(Batch *B) {
  if (B->br.empty()) {
    B->br.resize(B->nbr);
    B->join.resize(B->nbr);
    B->sets.resize(B->nbr, nullptr);
    for (int i = 0; i < B->nbr; i++) {
      if (cudaStreamCreateWithFlags(&B->br[i], cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&B->join[i], cudaEventDisableTiming) != cudaSuccess)
        return fail(E_CUDA, "batch: stream or event creation failed");
      B->sets[i] = scratch_set_create();
    }
    if (cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&B->origin, cudaStreamNonBlocking) != cudaSuccess)
      return fail(E_CUDA, "batch: stream or event creation failed");
  }
  std::vector<std::pair<double, int>> work;
  std::map<int, size_t> scratch_of_job;
  B->bytes = 0;
  for (auto &kv : B->jobs) {
    double w = 0;
    size_t sc = 0;
    for (auto &s : kv.second) {
      size_t ib = 0, ob = 0, sb = 0;
      int prec = 0;
      if (plan3d_sizes(s.plan, &ib, &ob, &sb, &prec) != E_OK) return E_BAD_ARG;
      w += (double)ib + (double)ob + 2.0 * sb;
      sc = std::max(sc, sb);
      B->bytes += (double)ib + (double)ob;
    }
    work.push_back({w, kv.first});
    scratch_of_job[kv.first] = sc;
  }
  std::sort(work.begin(), work.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
    return a.first > b.first || (a.first == b.first && a.second < b.second);
  });
  B->assign.assign(B->nbr, {});
  std::vector<double> load(B->nbr, 0.0);
  for (auto &w : work) {
    int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[k] += w.first;
    B->assign[k].push_back(w.second);
  }
  if (B->grouped) return E_OK;  // grouped mode gives every job its own scratch set instead
  for (int b = 0; b < B->nbr; b++) {
    size_t need = 0;
    for (int j : B->assign[b]) need = std::max(need, scratch_of_job[j]);
    if (need && scratch_set_reserve(B->sets[b], need) != E_OK) return E_CUDA;
  }
  return E_OK;
}

// Grouped mode.  Jobs with the same steps (plans and derivative directions) form a cohort; every
// job's stages are recorded with their buffers (each job has its own scratch set, since a
// cohort's jobs are in flight together), and for each stage the cohort's jobs run as ONE launch
// of the stage's specialised kernel over all their tiles.  Cohorts are independent: they are
// spread over the branch streams by longest-processing-time first, with no barrier between them.
// Measured on GB300: a shared launch helps jobs too small to fill the GPU (e.g. 16 x 64^3 FP64:
// 0.153 vs 0.160 ms) and costs large ones their overlap with other streams (8 x 256^3 FP32:
// 1.49 vs 1.24 ms), hence the size limit below.
static int prepare_grouped(Batch *B) {
  for (auto l : B->lsets) launch_set_destroy(l);
  B->lsets.clear();
  B->ngroups = 0;
  // record every job; its cohort key is the sequence of its stages' descriptions (kind, grids,
  // strides, precision, arithmetic, derivative) without the buffers, so equal plans made
  // separately still share launches
  std::map<std::vector<long long>, std::vector<std::pair<int, std::vector<StageLaunch>>>> cohorts;
  std::map<int, double> job_bytes;
  size_t js = 0;
  for (auto &kv : B->jobs) {
    if (js >= B->job_sets.size()) B->job_sets.push_back(scratch_set_create());
    std::vector<StageLaunch> rec;
    double w = 0;
    for (auto &s : kv.second) {
      const int rc = record_plan(s.plan, s.in, s.out, s.idir, B->job_sets[js], &rec);
      if (rc != E_OK) return rc;
      size_t ib = 0, ob = 0;
      plan3d_sizes(s.plan, &ib, &ob, nullptr, nullptr);
      w += (double)ib + (double)ob;
    }
    js++;
    std::vector<long long> key;
    for (auto &r : rec) {
      const StageDesc &d = r.d;
      for (long long v : {(long long)d.kind, (long long)d.r2r, (long long)d.prec, (long long)d.dt1, (long long)d.dt2,
                          (long long)d.L, (long long)d.deriv, (long long)d.engine, (long long)d.talt,
                          (long long)r.arith})
        key.push_back(v);
      for (int i = 0; i < 3; i++) {
        key.push_back(d.d1[i]);
        key.push_back(d.d2[i]);
        key.push_back(d.s1[i]);
        key.push_back(d.s2[i]);
      }
    }
    cohorts[key].push_back({kv.first, rec});
    job_bytes[kv.first] = w;
  }
  if (B->work_list) {
    // every job's k-th stage in level k; within a level, one work-list launch per kernel
    std::vector<std::vector<StageLaunch>> levels;
    B->level_jobs.clear();
    for (auto &c : cohorts)
      for (auto &jr : c.second) {
        if (levels.size() < jr.second.size()) {
          levels.resize(jr.second.size());
          B->level_jobs.resize(jr.second.size());
        }
        for (size_t k = 0; k < jr.second.size(); k++) {
          levels[k].push_back(jr.second[k]);
          B->level_jobs[k].push_back(jr.first);
        }
      }
    int err = E_OK;
    LaunchSet *ls = launch_set_build(levels, device_tables(), &err, true);
    if (!ls) return fail(err ? err : E_CUDA, "batch: work-list launch set could not be built");
    B->ngroups = launch_set_groups(ls);
    B->lsets.push_back(ls);
    size_t nitems = 0;
    for (int l = 0; l < launch_set_levels(ls); l++) nitems += (size_t)launch_set_items(ls, l);
    while (B->item_ev.size() < nitems) {
      cudaEvent_t e;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
        return fail(E_CUDA, "batch: event creation failed");
      B->item_ev.push_back(e);
    }
    return E_OK;
  }
  // Jobs large enough to fill the GPU on their own (>= 24 MB of steps' fields) gain nothing from a
  // shared launch and run better spread over the streams: they form cohorts of one.
  std::vector<std::vector<std::pair<int, std::vector<StageLaunch>>>> groups;
  for (auto &c : cohorts) {
    if (c.second.size() > 1 && job_bytes[c.second[0].first] >= 24.0 * (1 << 20)) {
      for (auto &jr : c.second) groups.push_back({jr});
    } else {
      groups.push_back(c.second);
    }
  }
  std::vector<std::pair<double, int>> work;
  for (auto &c : groups) {
    std::vector<std::vector<StageLaunch>> levels;
    double w = 0;
    for (auto &jr : c) {
      const std::vector<StageLaunch> &rec = jr.second;
      w += job_bytes[jr.first];
      if (levels.size() < rec.size()) levels.resize(rec.size());
      for (size_t k = 0; k < rec.size(); k++) levels[k].push_back(rec[k]);
    }
    int err = E_OK;
    LaunchSet *ls = launch_set_build(levels, device_tables(), &err);
    if (!ls) return fail(err ? err : E_CUDA, "batch: grouped launch set could not be built");
    B->ngroups += launch_set_groups(ls);
    work.push_back({w, (int)B->lsets.size()});
    B->lsets.push_back(ls);
  }
  std::sort(work.begin(), work.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
    return a.first > b.first || (a.first == b.first && a.second < b.second);
  });
  B->cassign.assign(B->nbr, {});
  std::vector<double> load(B->nbr, 0.0);
  for (auto &w : work) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[k] += w.first;
    B->cassign[k].push_back(w.second);
  }
  return E_OK;
}

// Work-list mode: the launches of a level go round-robin to the branch streams (largest first); a
// launch waits only for the launches that ran the previous stage of its own jobs.
static int run_work_list(Batch *B, cudaStream_t st) {
  LaunchSet *ls = B->lsets[0];
  int launched = 0, rc = E_OK;
  if (cudaEventRecord(B->fork, st) != cudaSuccess) return fail(E_CUDA, "batch: fork event failed");
  std::vector<char> used(B->nbr, 0);
  std::map<int, int> last;  // job -> event index of the launch that ran its latest stage
  int id = 0, rr = 0;
  for (int l = 0; l < launch_set_levels(ls) && rc == E_OK; l++) {
    for (int i = 0; i < launch_set_items(ls, l) && rc == E_OK; i++, id++) {
      const int b = rr++ % B->nbr;
      cudaStream_t s = B->br[b];
      if (!used[b]) {
        if (cudaStreamWaitEvent(s, B->fork, 0) != cudaSuccess) return fail(E_CUDA, "batch: fork wait failed");
        used[b] = 1;
      }
      std::vector<int> deps;
      for (int pos : launch_set_item_members(ls, l, i)) {
        auto it = last.find(B->level_jobs[l][pos]);
        if (it != last.end()) deps.push_back(it->second);
      }
      std::sort(deps.begin(), deps.end());
      deps.erase(std::unique(deps.begin(), deps.end()), deps.end());
      for (int d : deps)
        if (cudaStreamWaitEvent(s, B->item_ev[d], 0) != cudaSuccess) return fail(E_CUDA, "batch: dependency wait failed");
      rc = launch_set_run_item(ls, l, i, s, &launched);
      if (cudaEventRecord(B->item_ev[id], s) != cudaSuccess) return fail(E_CUDA, "batch: event record failed");
      for (int pos : launch_set_item_members(ls, l, i)) last[B->level_jobs[l][pos]] = id;
    }
  }
  // always join, so a failed capture still ends on the origin stream
  for (int b = 0; b < B->nbr; b++) {
    if (!used[b]) continue;
    if (cudaEventRecord(B->join[b], B->br[b]) != cudaSuccess || cudaStreamWaitEvent(st, B->join[b], 0) != cudaSuccess)
      return fail(E_CUDA, "batch: join failed");
  }
  add_kernel_count(launched);
  if (rc != E_OK) return fail(rc, "batch: work-list launch failed");
  return E_OK;
}

static int run_grouped(Batch *B, cudaStream_t st) {
  if (B->work_list) return run_work_list(B, st);
  int launched = 0, rc = E_OK;
  if (cudaEventRecord(B->fork, st) != cudaSuccess) return fail(E_CUDA, "batch: fork event failed");
  for (int b = 0; b < B->nbr; b++) {
    if (B->cassign[b].empty()) continue;
    if (cudaStreamWaitEvent(B->br[b], B->fork, 0) != cudaSuccess) return fail(E_CUDA, "batch: fork wait failed");
    for (int c : B->cassign[b])
      if (rc == E_OK) rc = launch_set_run(B->lsets[c], B->br[b], &launched);
    if (cudaEventRecord(B->join[b], B->br[b]) != cudaSuccess || cudaStreamWaitEvent(st, B->join[b], 0) != cudaSuccess)
      return fail(E_CUDA, "batch: join failed");
  }
  add_kernel_count(launched);
  if (rc != E_OK) return fail(rc, "batch: grouped launch failed");
  return E_OK;
}

// fork from `st`, run every branch's jobs, join back into `st`
static int run_branches(Batch *B, cudaStream_t st, bool capturing) {
  if (B->grouped) return run_grouped(B, st);
  if (cudaEventRecord(B->fork, st) != cudaSuccess) return fail(E_CUDA, "batch: fork event failed");
  int rc = E_OK;
  for (int b = 0; b < B->nbr; b++) {
    if (cudaStreamWaitEvent(B->br[b], B->fork, 0) != cudaSuccess) return fail(E_CUDA, "batch: fork wait failed");
    for (int j : B->assign[b]) {
      for (auto &s : B->jobs[j]) {
        rc = exec_plan_on(s.plan, s.in, s.out, s.idir, B->br[b], B->sets[b], capturing);
        if (rc != E_OK) break;
      }
      if (rc != E_OK) break;
    }
    // always join, so a failed capture still ends on the origin stream
    if (cudaEventRecord(B->join[b], B->br[b]) != cudaSuccess || cudaStreamWaitEvent(st, B->join[b], 0) != cudaSuccess)
      return fail(E_CUDA, "batch: join failed");
    if (rc != E_OK) return rc;
  }
  return E_OK;
}

static int build_graph(Batch *B) {
  if (B->gexec) {
    cudaGraphExecDestroy(B->gexec);
    B->gexec = nullptr;
  }
  const long long k0 = kernel_count_now();
  if (cudaStreamBeginCapture(B->origin, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return fail(E_CUDA, "batch: stream capture could not begin");
  int rc = run_branches(B, B->origin, true);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(B->origin, &graph);
  add_kernel_count(-(kernel_count_now() - k0));  // recorded, not launched
  if (rc != E_OK || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return rc != E_OK ? rc : fail(E_CUDA, "batch: stream capture failed");
  }
  e = cudaGraphInstantiate(&B->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    B->gexec = nullptr;
    cudaGetLastError();
    return fail(E_CUDA, "batch: graph instantiation failed");
  }
  return E_OK;
}

static int finish(cudaStream_t st) {
  if (!library_sync()) return E_OK;
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(E_CUDA, cudaGetErrorString(e));
  return E_OK;
}

}  // namespace p3d

using namespace p3d;

extern "C" {

int p3dfft_gb300_batch_create(int nbranches) {
  if (nbranches < 0 || nbranches > 64) {
    record_error(E_BAD_ARG, "batch: branch count must be 0 (default 8) .. 64");
    return -1;
  }
  Batch *B = new Batch();
  B->nbr = nbranches ? nbranches : 8;
  std::lock_guard<std::mutex> g(g_bmu);
  g_batches.push_back(B);
  return (int)g_batches.size() - 1;
}

int p3dfft_gb300_batch_add(int batch, int job, int plan, const void *in, void *out, int idir) {
  Batch *B = get_batch(batch);
  if (!B) return fail(E_BAD_ARG, "batch: invalid handle");
  if (job < 0) return fail(E_BAD_ARG, "batch: job ids are >= 0");
  if (idir > 2) return fail(E_BAD_ARG, "batch: derivative direction out of range");
  if (!in || !out) return fail(E_BAD_ARG, "batch: null data pointer");
  if (plan3d_sizes(plan, nullptr, nullptr, nullptr, nullptr) != E_OK) return E_BAD_ARG;
  cudaPointerAttributes a1, a2;
  if (cudaPointerGetAttributes(&a1, in) != cudaSuccess || cudaPointerGetAttributes(&a2, out) != cudaSuccess ||
      a1.type != cudaMemoryTypeDevice || a2.type != cudaMemoryTypeDevice) {
    cudaGetLastError();
    return fail(E_BAD_ARG, "batch: jobs take device pointers only");
  }
  B->jobs[job].push_back({plan, in, out, idir});
  B->dirty = true;
  return E_OK;
}

int p3dfft_gb300_batch_set_graph(int batch, int on) {
  Batch *B = get_batch(batch);
  if (!B) return fail(E_BAD_ARG, "batch: invalid handle");
  B->use_graph = on != 0;
  B->dirty = true;
  return E_OK;
}

int p3dfft_gb300_batch_set_grouped(int batch, int on) {
  Batch *B = get_batch(batch);
  if (!B) return fail(E_BAD_ARG, "batch: invalid handle");
  B->grouped = on != 0;
  B->work_list = on == 2;
  B->dirty = true;
  return E_OK;
}

int p3dfft_gb300_batch_groups(int batch) {
  Batch *B = get_batch(batch);
  return B ? (B->grouped ? B->ngroups : 0) : -1;
}

int p3dfft_gb300_batch_exec(int batch) {
  Batch *B = get_batch(batch);
  if (!B) return fail(E_BAD_ARG, "batch: invalid handle");
  if (!device_ready()) return E_NO_DEVICE;
  if (B->jobs.empty()) return E_OK;
  const cudaStream_t st = library_stream();
  const int ar = current_arith();
  if (B->dirty || ar != B->arith || (B->use_graph && !B->gexec)) {
    int rc = prepare(B);
    if (rc != E_OK) return rc;
    if (B->grouped) {
      rc = prepare_grouped(B);
      if (rc != E_OK) return rc;
    }
    const long long k0 = kernel_count_now();
    rc = run_branches(B, st, false);  // eager run: resolves tables, produces this call's results
    if (rc != E_OK) return rc;
    B->kernels = kernel_count_now() - k0;
    if (B->use_graph) {
      rc = build_graph(B);
      if (rc != E_OK) return rc;
    }
    B->dirty = false;
    B->arith = ar;
    return finish(st);
  }
  if (B->use_graph) {
    if (cudaGraphLaunch(B->gexec, st) != cudaSuccess) return fail(E_CUDA, "batch: graph launch failed");
    add_kernel_count(B->kernels);
  } else {
    int rc = run_branches(B, st, false);
    if (rc != E_OK) return rc;
  }
  return finish(st);
}

long long p3dfft_gb300_batch_kernels(int batch) {
  Batch *B = get_batch(batch);
  return B ? B->kernels : -1;
}

double p3dfft_gb300_batch_field_bytes(int batch) {
  Batch *B = get_batch(batch);
  return B ? B->bytes : -1.0;
}

int p3dfft_gb300_batch_destroy(int batch) {
  Batch *B;
  {
    std::lock_guard<std::mutex> g(g_bmu);
    if (batch < 0 || batch >= (int)g_batches.size() || !g_batches[batch]) return E_BAD_ARG;
    B = g_batches[batch];
    g_batches[batch] = nullptr;
  }
  cudaStreamSynchronize(library_stream());
  delete B;
  return E_OK;
}

}  // extern "C"
