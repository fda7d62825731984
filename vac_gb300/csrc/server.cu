// server.cu - continuous-batching request server for TVDLF solves.
//
// Requests (a grid, its initial state and a step count) arrive at any time
// from any host thread.  A worker thread admits queued requests while the
// device-memory budget and the slot limit allow, keeps every admitted
// request's state resident on the device, and keeps each one moving by
// issuing chunks of steps (replayed CUDA graphs) on the request's own
// stream as soon as its previous chunk has finished -- so the work of all
// admitted requests overlaps on the GPU and a newly admitted request starts
// while earlier ones are still running.  A finished request's state is
// copied back, its device memory released, and the slot handed to the next
// request.  Time-to-solution is measured from submission to the moment the
// result is on the host.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/vacgpu.h"

int vacgpu_internal_fail(const char* msg);
int vacgpu_internal_step_async(vacgpu_handle* h, int k);
void* vacgpu_internal_stream(vacgpu_handle* h);
size_t vacgpu_internal_device_bytes(const vacgpu_params* p);

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
  long long id;
  vacgpu_params p;
  std::vector<double> x, w;
  int nsteps;
  double t_submit;
  double t_admit = 0.0;  // device work (allocation, upload) begins
  size_t bytes;
  vacgpu_handle* h = nullptr;
  cudaEvent_t ev = nullptr;
  int issued = 0;
  int state = 0;  // 0 queued, 1 active, 2 done, 3 failed
  std::vector<double> result;
  double t_done = 0.0, t_sim = 0.0;
  int it = 0;
  std::string err;
  long long cells = 0;
};

}  // namespace

struct vacgpu_server {
  double budget;
  int max_active;
  int chunk;
  size_t used = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Req*> queue;
  std::vector<Req*> active;
  std::map<long long, Req*> all;
  std::thread worker;
  bool stop = false;
  long long next_id = 1;
  int device = 0;
  double cell_updates_done = 0.0;
  double t_first = -1.0, t_last = -1.0;
  int peak_active = 0;
  std::atomic<int> nact{0};
};

namespace {

void finish(vacgpu_server* s, Req* r, bool ok, const std::string& err) {
  if (ok) {
    r->result.resize(r->w.size());
    double dt;
    int fin;
    if (vacgpu_step(r->h, 0, 1e300, &r->t_sim, &r->it, &dt, &fin) ||
        vacgpu_download(r->h, r->result.data())) {
      ok = false;
      char buf[512];
      vacgpu_last_error(buf, sizeof buf);
      r->err = buf;
    }
  }
  if (r->ev) cudaEventDestroy(r->ev);
  if (r->h) vacgpu_destroy(r->h);
  r->h = nullptr;
  r->ev = nullptr;
  std::lock_guard<std::mutex> lk(s->mu);
  s->used -= r->bytes;
  r->t_done = now_s();
  if (!ok && r->err.empty()) r->err = err;
  r->state = ok ? 2 : 3;
  if (ok) {
    s->cell_updates_done += (double)r->cells * r->nsteps;
    s->t_last = r->t_done;
  }
  r->x.clear();
  r->x.shrink_to_fit();
  r->w.clear();
  r->w.shrink_to_fit();
  s->cv.notify_all();
}

bool admit_one(Req* r) {
  char buf[512];
  r->t_admit = now_s();
  if (vacgpu_create(&r->p, &r->h) || vacgpu_set_grid(r->h, r->x.data()) ||
      vacgpu_upload(r->h, r->w.data(), 0, 0.0)) {
    vacgpu_last_error(buf, sizeof buf);
    r->err = buf;
    return false;
  }
  if (cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming) != cudaSuccess) {
    r->err = "event creation failed";
    return false;
  }
  return true;
}

void worker_loop(vacgpu_server* s) {
  cudaSetDevice(s->device);
  while (true) {
    // admission: FIFO, within the memory budget and the slot limit
    std::vector<Req*> admit;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop) break;
      if (s->queue.empty() && s->active.empty()) {
        s->cv.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
      while (!s->queue.empty() &&
             (int)(s->active.size() + admit.size()) < s->max_active) {
        Req* r = s->queue.front();
        if ((double)(s->used + r->bytes) > s->budget &&
            !(s->active.empty() && admit.empty()))
          break;  // wait for memory (a lone oversized request still runs)
        s->queue.pop_front();
        s->used += r->bytes;
        admit.push_back(r);
      }
    }
    for (Req* r : admit) {
      if (!admit_one(r)) {
        finish(s, r, false, r->err);
        continue;
      }
      r->state = 1;
      s->active.push_back(r);
      s->nact = (int)s->active.size();
      if ((int)s->active.size() > s->peak_active) s->peak_active = (int)s->active.size();
    }
    // keep every admitted request moving
    bool progressed = false;
    for (size_t i = 0; i < s->active.size();) {
      Req* r = s->active[i];
      const bool idle = r->issued == 0 || cudaEventQuery(r->ev) == cudaSuccess;
      if (!idle) {
        i++;
        continue;
      }
      progressed = true;
      if (r->issued < r->nsteps) {
        const int k = r->nsteps - r->issued < s->chunk ? r->nsteps - r->issued : s->chunk;
        if (vacgpu_internal_step_async(r->h, k) ||
            cudaEventRecord(r->ev, (cudaStream_t)vacgpu_internal_stream(r->h)) !=
                cudaSuccess) {
          char buf[512];
          vacgpu_last_error(buf, sizeof buf);
          s->active.erase(s->active.begin() + i);
          s->nact = (int)s->active.size();
          finish(s, r, false, buf);
          continue;
        }
        r->issued += k;
        i++;
      } else {
        s->active.erase(s->active.begin() + i);
        s->nact = (int)s->active.size();
        finish(s, r, true, "");
      }
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  for (Req* r : s->active) {
    if (r->ev) cudaEventDestroy(r->ev);
    if (r->h) vacgpu_destroy(r->h);
  }
  s->active.clear();
}

}  // namespace

extern "C" {

int vacgpu_server_create(double hbm_budget_bytes, int max_active,
                         int steps_per_chunk, vacgpu_server** out) {
  *out = nullptr;
  if (!(hbm_budget_bytes > 0) || max_active < 1 || steps_per_chunk < 1)
    return vacgpu_internal_fail("server: bad budget, slot count or chunk");
  vacgpu_server* s = new vacgpu_server();
  s->budget = hbm_budget_bytes;
  s->max_active = max_active;
  s->chunk = steps_per_chunk;
  cudaGetDevice(&s->device);
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return 0;
}

int vacgpu_server_submit(vacgpu_server* s, const vacgpu_params* p,
                         const double* x, const double* w, int nsteps,
                         long long* id) {
  const double t0 = now_s();
  if (!s || !p || !x || !w || nsteps < 1)
    return vacgpu_internal_fail("server: bad submission");
  long long ncell = 1;
  for (int d = 0; d < p->ndim; d++) ncell *= p->nx[d];
  Req* r = new Req();
  r->p = *p;
  r->p.itmax = 1000000000;  // the request's own step count bounds the run
  r->p.tmax = 1e99;
  r->x.assign(x, x + (size_t)ncell * p->ndim);
  r->w.assign(w, w + (size_t)ncell * p->nw);
  r->nsteps = nsteps;
  r->cells = ncell;
  r->bytes = vacgpu_internal_device_bytes(p);
  std::lock_guard<std::mutex> lk(s->mu);
  r->id = s->next_id++;
  r->t_submit = t0;
  if (s->t_first < 0) s->t_first = r->t_submit;
  s->all[r->id] = r;
  s->queue.push_back(r);
  s->cv.notify_all();
  *id = r->id;
  return 0;
}

// 0: done (result copied when w is not NULL); 1: still queued or running
// (after waiting up to wait_s seconds); other nonzero: the request failed.
int vacgpu_server_result(vacgpu_server* s, long long id, double wait_s,
                         double* w, double* t, int* it, double* tts) {
  if (!s) return vacgpu_internal_fail("null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto f = s->all.find(id);
  if (f == s->all.end()) return vacgpu_internal_fail("unknown request id");
  Req* r = f->second;
  if (wait_s > 0 && r->state < 2)
    s->cv.wait_for(lk, std::chrono::duration<double>(wait_s),
                   [&] { return r->state >= 2; });
  if (r->state == 3) return vacgpu_internal_fail(("request failed: " + r->err).c_str());
  if (r->state < 2) return 1;
  if (w) memcpy(w, r->result.data(), r->result.size() * sizeof(double));
  if (t) *t = r->t_sim;
  if (it) *it = r->it;
  if (tts) *tts = r->t_done - r->t_submit;
  return 0;
}

int vacgpu_server_timing(vacgpu_server* s, long long id, double* queue_s,
                         double* service_s) {
  if (!s) return vacgpu_internal_fail("null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto f = s->all.find(id);
  if (f == s->all.end()) return vacgpu_internal_fail("unknown request id");
  Req* r = f->second;
  if (r->state < 2) return 1;
  if (queue_s) *queue_s = r->t_admit - r->t_submit;
  if (service_s) *service_s = r->t_done - r->t_admit;
  return 0;
}

int vacgpu_server_stats(vacgpu_server* s, int* nqueued, int* nactive,
                        int* ndone, int* peak_active, double* cell_updates,
                        double* span_s) {
  if (!s) return vacgpu_internal_fail("null server");
  std::lock_guard<std::mutex> lk(s->mu);
  int done = 0;
  for (auto& kv : s->all) done += kv.second->state == 2;
  if (nqueued) *nqueued = (int)s->queue.size();
  if (nactive) *nactive = s->nact.load();
  if (ndone) *ndone = done;
  if (peak_active) *peak_active = s->peak_active;
  if (cell_updates) *cell_updates = s->cell_updates_done;
  if (span_s) *span_s = s->t_last > s->t_first ? s->t_last - s->t_first : 0.0;
  return 0;
}

void vacgpu_server_destroy(vacgpu_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (auto& kv : s->all) delete kv.second;
  delete s;
}

}  // extern "C"
