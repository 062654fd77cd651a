// serve.cpp — the request server (eik_server_*): resident pool meshes, admission
// into instance slots, continuous batching on one device loop per dimension.
//
// Threads: callers submit and poll under one mutex; one worker thread per arena
// (2D, 3D) owns that arena's DeviceSolve and CUDA stream.  A worker loop:
//   1. admit queued requests whose mesh has a free slot (arrival order),
//   2. run the serving graph: outer iterations over every running instance until
//      one finishes or a newly submitted request raises the pending flag,
//   3. read which instances finished, copy their travel times to pinned memory,
//      complete those requests and free their slots.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/eikonal_gb300.h"
#include "device.hpp"
#include "setup.hpp"
#include "solver_access.hpp"

using namespace eikgb;

namespace {

struct PoolMesh {
  MeshSnapshot snap;
  int slots_req = 0;
  int slots = 0;
  size_t bytes = 0;          // device bytes of one slot
  int arena = -1;            // 0: 2D, 1: 3D
  int local = -1;            // index among the arena's meshes
};

struct Request {
  long long id = 0;
  int mesh = 0;
  std::vector<int> seeds;
  float scale = 1.0f;
  double t_submit = 0, t_admit = 0;
  int inst = -1;
  bool cancelled = false;
};

struct Arena {
  int dim = 0;
  bool used = false;
  Layout L;
  std::unique_ptr<DeviceSolve> dev;
  std::vector<int> inst_mesh;                 // global pool mesh id per instance
  std::vector<std::vector<int>> free_slots;   // per global mesh id
  std::vector<long long> inst_req;            // running request per instance, -1 idle
  std::unordered_map<long long, Request> running;
  volatile int* pending = nullptr;
  std::thread worker;
  long long loops = 0;
  size_t bytes = 0;
  double busy_s = 0;
  long long updates = 0;
};

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

float coef_scale(int dim, float s) {
  // 2D: speeds times s; 3D: metric (inverse squared speed) times 1/s^2
  return (dim == 2) ? s : (float)(1.0 / ((double)s * (double)s));
}

}  // namespace

struct eik_server {
  long long budget = 0;
  int max_inflight = 0;
  bool keep = false;
  std::vector<PoolMesh> meshes;
  Arena arenas[2];
  bool started = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request> queue;
  std::unordered_set<long long> cancel_running;  // running requests to stop
  long long next_id = 1;
  int inflight = 0;
  bool stop = false;
  int failed = EIK_OK;
  std::deque<eik_completion> done;
  std::unordered_map<long long, std::vector<float>> results;
  long long submitted = 0, completed = 0;
  std::string err;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
};

namespace {

bool admissible(const eik_server* S, const Request& r) {
  const PoolMesh& m = S->meshes[r.mesh];
  const Arena& A = S->arenas[m.arena];
  if (A.free_slots[r.mesh].empty()) return false;
  return S->max_inflight <= 0 || S->inflight < S->max_inflight;
}

bool has_admissible(const eik_server* S, int ai) {
  for (const Request& r : S->queue)
    if (S->meshes[r.mesh].arena == ai && admissible(S, r)) return true;
  return false;
}

// Raise the pending flag of every arena that could admit a queued request now.
void signal_arenas(eik_server* S) {
  for (int ai = 0; ai < 2; ++ai) {
    Arena& A = S->arenas[ai];
    if (A.used && A.pending && has_admissible(S, ai)) *A.pending = 1;
  }
  S->cv_work.notify_all();
}

void fail_running(eik_server* S, Arena& A, int code, double t) {
  for (auto& kv : A.running) {
    const Request& r = kv.second;
    eik_completion c{};
    c.id = r.id;
    c.mesh = r.mesh;
    c.status = code;
    c.submit_s = r.t_submit;
    c.admit_s = r.t_admit;
    c.done_s = t;
    S->done.push_back(c);
    S->inflight--;
    S->completed++;
  }
  A.running.clear();
}

// Completes every queued and running request with `code` (the server stops).
void fail_all(eik_server* S, int code, double t) {
  for (Arena& A : S->arenas) fail_running(S, A, code, t);
  for (const Request& r : S->queue) {
    eik_completion c{};
    c.id = r.id;
    c.mesh = r.mesh;
    c.status = code;
    c.submit_s = r.t_submit;
    c.done_s = t;
    S->done.push_back(c);
    S->completed++;
  }
  S->queue.clear();
}

void worker_loop(eik_server* S, int ai) {
  Arena& A = S->arenas[ai];
  A.dev->bind_thread();
  std::vector<int> done, iters;
  for (;;) {
    std::vector<Admission> adm;
    std::vector<int> cancel;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stop || !A.running.empty() || has_admissible(S, ai); });
      if (S->stop) return;
      for (auto& kv : A.running)
        if (!kv.second.cancelled && S->cancel_running.count(kv.first)) {
          kv.second.cancelled = true;
          S->cancel_running.erase(kv.first);
          cancel.push_back(kv.second.inst);
        }
      for (auto it = S->queue.begin(); it != S->queue.end();) {
        if (S->meshes[it->mesh].arena != ai || !admissible(S, *it)) {
          ++it;
          continue;
        }
        Request r = std::move(*it);
        it = S->queue.erase(it);
        const int inst = A.free_slots[r.mesh].back();
        A.free_slots[r.mesh].pop_back();
        Admission x;
        x.inst = inst;
        x.coef_scale = coef_scale(A.dim, r.scale);
        x.max_iterations = S->meshes[r.mesh].snap.max_iterations;
        x.seeds = r.seeds;
        adm.push_back(std::move(x));
        r.inst = inst;
        r.t_admit = seconds_since(S->t0);
        A.inst_req[inst] = r.id;
        S->inflight++;
        A.running.emplace(r.id, std::move(r));
      }
      *A.pending = 0;
    }
    std::string e;
    const auto r0 = std::chrono::steady_clock::now();
    if (!cancel.empty()) e = A.dev->serve_cancel(cancel);
    if (e.empty() && !adm.empty()) e = A.dev->serve_admit(adm);
    if (e.empty()) e = A.dev->serve_run();
    const double run_s = seconds_since(r0);
    if (e.empty()) e = A.dev->serve_poll(done, iters);
    std::vector<int> fin;
    if (e.empty()) {
      for (size_t i = 0; i < A.inst_req.size(); ++i)
        if (A.inst_req[i] >= 0 && done[i]) fin.push_back((int)i);
      for (int i : fin)
        if (e.empty()) e = A.dev->serve_fetch(i);
      if (e.empty()) e = A.dev->serve_sync();
    }
    const double t = seconds_since(S->t0);
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return;  // the other arena failed: its worker completed everything
    A.loops++;
    A.busy_s += run_s;
    A.updates = A.dev->stats().vertex_updates;
    if (!e.empty()) {
      S->err = "device loop (" + std::string(A.dim == 2 ? "2D" : "3D") + "): " + e;
      S->failed = EIK_ERR_CUDA;
      fail_all(S, EIK_ERR_CUDA, t);
      S->stop = true;
      S->cv_work.notify_all();
      S->cv_done.notify_all();
      return;
    }
    for (int i : fin) {
      auto it = A.running.find(A.inst_req[i]);
      Request& r = it->second;
      eik_completion c{};
      c.id = r.id;
      c.mesh = r.mesh;
      c.iterations = iters[i];
      c.status = r.cancelled ? EIK_ERR_CANCELLED : EIK_OK;
      c.submit_s = r.t_submit;
      c.admit_s = r.t_admit;
      c.done_s = t;
      if (S->keep && !r.cancelled) {
        const float* p = A.dev->serve_host_result(i);
        S->results[r.id].assign(p, p + S->meshes[r.mesh].snap.nv);
      }
      S->done.push_back(c);
      S->cancel_running.erase(r.id);
      A.free_slots[r.mesh].push_back(i);
      A.inst_req[i] = -1;
      A.running.erase(it);
      S->inflight--;
      S->completed++;
    }
    if (!fin.empty()) {
      S->cv_done.notify_all();
      signal_arenas(S);
    }
  }
}

int sfail(eik_server* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}

}  // namespace

extern "C" {

int eik_server_create(long long hbm_budget_bytes, int max_inflight, int keep_results, eik_server** out) {
  if (!out) return EIK_ERR_ARG;
  *out = nullptr;
  if (hbm_budget_bytes < 0 || max_inflight < 0) return EIK_ERR_ARG;
  eik_server* s = new eik_server;
  s->budget = hbm_budget_bytes;
  s->max_inflight = max_inflight;
  s->keep = keep_results != 0;
  *out = s;
  return EIK_OK;
}

int eik_server_add_mesh(eik_server* s, eik_solver* h, int slots, int* mesh_id) {
  if (!s || !h || slots < 0) return EIK_ERR_ARG;
  if (s->started) return sfail(s, EIK_ERR_STATE, "meshes are added before eik_server_start");
  PoolMesh m;
  std::string e;
  int rc = snapshot_for_server(h, m.snap, e);
  if (rc) return sfail(s, rc, e);
  m.slots_req = slots;
  m.bytes = device_footprint(m.snap.layout, m.snap.built.get());
  m.arena = (m.snap.dim == 2) ? 0 : 1;
  s->meshes.push_back(std::move(m));
  if (mesh_id) *mesh_id = (int)s->meshes.size() - 1;
  return EIK_OK;
}

int eik_server_mesh_info(const eik_server* s, int mesh_id, int* nv, int* slots, long long* device_bytes) {
  if (!s || mesh_id < 0 || mesh_id >= (int)s->meshes.size()) return EIK_ERR_ARG;
  const PoolMesh& m = s->meshes[mesh_id];
  if (nv) *nv = m.snap.nv;
  if (slots) *slots = m.slots;
  if (device_bytes) *device_bytes = (long long)m.bytes;
  return EIK_OK;
}

int eik_server_start(eik_server* s) {
  if (!s) return EIK_ERR_ARG;
  if (s->started) return sfail(s, EIK_ERR_STATE, "server already started");
  if (s->meshes.empty()) return sfail(s, EIK_ERR_STATE, "no pool meshes");
  // slots per mesh from the budget
  int nauto = 0;
  long long fixed = 0;
  for (const PoolMesh& m : s->meshes) {
    if (m.slots_req == 0) ++nauto;
    else fixed += (long long)m.slots_req * (long long)m.bytes;
  }
  const long long share = nauto ? std::max(0ll, (s->budget - fixed) / nauto) : 0;
  long long need = 0;
  for (PoolMesh& m : s->meshes) {
    if (m.slots_req > 0) m.slots = m.slots_req;
    else m.slots = (int)std::min<long long>(64, std::max<long long>(1, share / (long long)std::max<size_t>(m.bytes, 1)));
    need += (long long)m.slots * (long long)m.bytes;
  }
  if (s->budget > 0 && need > s->budget)
    return sfail(s, EIK_ERR_LIMIT, "the pool's slots need " + std::to_string(need) + " device bytes, over the budget of " +
                                       std::to_string(s->budget));
  for (int ai = 0; ai < 2; ++ai) {
    Arena& A = s->arenas[ai];
    A.dim = ai == 0 ? 2 : 3;
    std::vector<const Layout*> parts;
    std::vector<ServeSource> src;
    std::vector<int> local_mesh;
    A.free_slots.assign(s->meshes.size(), {});
    int sweeps = -1, threads = 0;
    for (size_t mi = 0; mi < s->meshes.size(); ++mi) {
      PoolMesh& m = s->meshes[mi];
      if (m.arena != ai) continue;
      if (!A.used) {
        sweeps = m.snap.fim_sweeps;
        threads = m.snap.threads;
      }
      A.used = true;
      m.local = (int)src.size();
      ServeSource x;
      x.dim = m.snap.dim;
      x.nv = m.snap.nv;
      if (x.dim == 3) {
        x.xyz = m.snap.xyz.data();
        x.tets = m.snap.elems.data();
        x.nt = m.snap.ne;
        x.M6 = m.snap.M6.data();
      } else {
        x.speed = m.snap.speed.data();
        x.nf = m.snap.ne;
      }
      src.push_back(x);
      for (int k = 0; k < m.slots; ++k) {
        A.free_slots[mi].push_back((int)parts.size());
        A.inst_mesh.push_back((int)mi);
        local_mesh.push_back(m.local);
        parts.push_back(&m.snap.layout);
      }
      std::reverse(A.free_slots[mi].begin(), A.free_slots[mi].end());
      A.bytes += (size_t)m.slots * m.bytes;
    }
    if (!A.used) continue;
    // pool meshes built on the device are replicated there; an arena that also
    // holds host-built meshes is concatenated on the host
    bool all_built = true;
    for (const PoolMesh& m : s->meshes)
      if (m.arena == ai && !m.snap.built) all_built = false;
    std::string e;
    A.dev.reset(new DeviceSolve);
    if (all_built) {
      std::vector<const Built3D*> bparts;
      std::vector<int> nhalo;
      for (int mi : A.inst_mesh) {
        bparts.push_back(s->meshes[mi].snap.built.get());
        nhalo.push_back(s->meshes[mi].snap.built->nhalo);
      }
      e = concat_layout_headers(parts, nhalo, A.L);
      if (!e.empty()) return sfail(s, EIK_ERR_ARG, e);
      e = A.dev->upload_replicas(A.L, bparts);
    } else {
      for (PoolMesh& m : s->meshes)
        if (m.arena == ai && m.snap.built) {
          e = download_built(*m.snap.built, m.snap.layout);
          if (!e.empty()) return sfail(s, EIK_ERR_CUDA, e);
          m.snap.built.reset();
        }
      e = concat_layouts(parts, A.L);
      if (!e.empty()) return sfail(s, EIK_ERR_ARG, e);
      e = A.dev->upload(A.L);
    }
    if (!e.empty()) return sfail(s, e.find("shared memory") != std::string::npos ? EIK_ERR_LIMIT : EIK_ERR_CUDA, e);
    e = A.dev->serve_setup(src, local_mesh, sweeps, threads);
    if (!e.empty()) return sfail(s, EIK_ERR_CUDA, e);
    for (PoolMesh& m : s->meshes)
      if (m.arena == ai) m.snap.built.reset();  // replicated: the arena holds the arrays now
    A.inst_req.assign(parts.size(), -1);
    A.pending = A.dev->serve_pending();
  }
  s->started = true;
  for (int ai = 0; ai < 2; ++ai)
    if (s->arenas[ai].used) s->arenas[ai].worker = std::thread(worker_loop, s, ai);
  return EIK_OK;
}

int eik_server_submit(eik_server* s, int mesh_id, const int* seeds, int nseeds, float speed_scale, long long* id) {
  if (!s) return EIK_ERR_ARG;
  if (mesh_id < 0 || mesh_id >= (int)s->meshes.size()) return sfail(s, EIK_ERR_ARG, "pool mesh id out of range");
  if (!seeds || nseeds <= 0) return sfail(s, EIK_ERR_ARG, "a request needs at least one seed vertex");
  if (!(speed_scale > 0.0f) || speed_scale > 1e30f) return sfail(s, EIK_ERR_ARG, "speed scale must be positive");
  const int nv = s->meshes[mesh_id].snap.nv;
  for (int i = 0; i < nseeds; ++i)
    if (seeds[i] < 0 || seeds[i] >= nv) return sfail(s, EIK_ERR_ARG, "seed out of range");
  std::lock_guard<std::mutex> lk(s->mu);
  if (!s->started) return sfail(s, EIK_ERR_STATE, "server not started");
  if (s->failed) return sfail(s, s->failed, s->err);
  Request r;
  r.id = s->next_id++;
  r.mesh = mesh_id;
  r.seeds.assign(seeds, seeds + nseeds);
  r.scale = speed_scale;
  r.t_submit = seconds_since(s->t0);
  if (id) *id = r.id;
  s->queue.push_back(std::move(r));
  s->submitted++;
  signal_arenas(s);
  return EIK_OK;
}

int eik_server_poll(eik_server* s, eik_completion* out, int max, int wait_ms, int* n) {
  if (!s || !n || (max > 0 && !out)) return EIK_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && wait_ms > 0)
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty() || s->stop; });
  int k = 0;
  while (k < max && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *n = k;
  return s->failed;
}

int eik_server_result(eik_server* s, long long id, float* out, int nv) {
  if (!s || !out) return EIK_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->results.find(id);
  if (it == s->results.end()) return sfail(s, EIK_ERR_STATE, "no kept result for this request");
  if ((int)it->second.size() != nv) return sfail(s, EIK_ERR_ARG, "size mismatch");
  std::memcpy(out, it->second.data(), sizeof(float) * (size_t)nv);
  s->results.erase(it);
  return EIK_OK;
}

int eik_server_cancel(eik_server* s, long long id) {
  if (!s) return EIK_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
    if (it->id != id) continue;
    eik_completion c{};
    c.id = it->id;
    c.mesh = it->mesh;
    c.status = EIK_ERR_CANCELLED;
    c.submit_s = it->t_submit;
    c.done_s = seconds_since(s->t0);
    s->done.push_back(c);
    s->completed++;
    s->queue.erase(it);
    s->cv_done.notify_all();
    return EIK_OK;
  }
  for (Arena& A : s->arenas)
    if (A.running.count(id)) {
      s->cancel_running.insert(id);
      if (A.pending) *A.pending = 1;  // end the device loop after this iteration
      s->cv_work.notify_all();
      return EIK_OK;
    }
  return sfail(s, EIK_ERR_ARG, "no queued or running request with this id");
}

int eik_server_drain(eik_server* s, int timeout_ms) {
  if (!s) return EIK_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto idle = [&] { return (s->queue.empty() && s->inflight == 0) || s->stop; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, idle);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle)) {
    return sfail(s, EIK_ERR_STATE, "timed out with requests still queued or running");
  }
  return s->failed;
}

int eik_server_get_stats(eik_server* s, eik_server_stats* out) {
  if (!s || !out) return EIK_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->queued = (long long)s->queue.size();
  out->running = s->inflight;
  out->device_bytes = (long long)(s->arenas[0].bytes + s->arenas[1].bytes);
  out->slots_2d = (int)s->arenas[0].inst_req.size();
  out->slots_3d = (int)s->arenas[1].inst_req.size();
  out->device_loops = s->arenas[0].loops + s->arenas[1].loops;
  for (int i = 0; i < 2; ++i) {
    out->busy_s[i] = s->arenas[i].busy_s;
    out->vertex_updates[i] = s->arenas[i].updates;
  }
  return EIK_OK;
}

void eik_server_destroy(eik_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (Arena& A : s->arenas)
      if (A.pending) *A.pending = 1;
  }
  s->cv_work.notify_all();
  s->cv_done.notify_all();
  for (Arena& A : s->arenas)
    if (A.worker.joinable()) A.worker.join();
  delete s;
}

const char* eik_server_last_error(const eik_server* s) { return s ? s->err.c_str() : "null handle"; }

}  // extern "C"
