// Serving loop: continuous batching of k-NN requests over resident indexes.
//
// No reference counterpart (the reference answers one batch per process run).  Design:
//  * submit() copies the request, checks admission (queue capacity, and enough free HBM
//    above a reserve for the request's buffers) and enqueues it;
//  * one scheduler thread owns `streams` launch slots.  Whenever a slot is free it takes
//    the oldest pending request whose index holds fewer than streams - 1 busy slots while
//    requests for other indexes wait (so long requests on one index cannot occupy every
//    slot) and coalesces the following
//    requests for the same index and candidate class up to max_batch queries; a batch of
//    fewer than max_batch queries waits until its oldest request is batch_window_us old,
//    so that requests arriving meanwhile join it.  Requests with different k share a
//    launch when the index computes the same candidates for them (batch_class): the
//    launch runs at the largest k and each request receives the first k of its rows,
//    which is its own top-k: the lists are sorted, ties by lower index, and the FP64
//    re-check orders the near-ties around the k-th place of every k in the launch (at most
//    four distinct k a launch; their list is copied to the device before each launch, so
//    the recorded graph of the largest k serves every mix).  The batch is padded to a power-of-two
//    class by repeating its last query, copied into the slot's pinned buffer and launched;
//    requests that arrive while other batches are on the GPU go to the next free slot, so
//    their work overlaps on the device;
//  * each (slot, index, k, class) launch is recorded once into a CUDA graph and replayed
//    afterwards (falling back to direct launches if recording fails);
//  * a host callback at the end of each slot's stream wakes the scheduler, which splits
//    the results back into the requests and stamps their completion time.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <functional>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "index.h"

using namespace lshg;

namespace lshg {
void set_last_error(const char* msg);
}

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  int index_id = 0;
  int nq = 0, k = 0;
  std::vector<float> q;
  std::vector<lshg_point> out;
  Clock::time_point t_submit, t_done;
  int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
  int status = LSHG_OK;
  std::string err;
};

// Requests whose (index, class) match get the same candidates whatever their k, so they
// can share a launch run at the largest k.  The BF16 tensor-core scan re-ranks 64
// candidates for k <= 32 and 128 beyond, the E4M3 one 128 always; sketched scans max(C, k rounded up); exact scans and LSH
// buckets do not depend on k.
int batch_class(const Index& I, int k) {
  const int impl = I.p.implementation == 1 ? 2 : I.p.implementation;
  if (I.p.framework == 0 && impl == 8) return k <= 32 ? 0 : 1;
  if (I.p.framework == 0 && impl == 9) return 0;  // 128 candidates at every k
  int kp = 32;
  while (kp < k) kp <<= 1;
  const bool sketched =
      I.p.framework == 0 ? ((impl >= 3 && impl <= 6) || impl == 10) : (I.p.runWithSketchedData && I.sk_kind);
  if (sketched) return std::max(I.C, kp);
  return 0;
}

struct Slot {
  cudaStream_t stream = nullptr;
  float* h_in = nullptr;
  float* d_in = nullptr;
  lshg_point* h_out = nullptr;
  lshg_point* d_out = nullptr;
  size_t in_cap = 0, out_cap = 0;  // elements
  bool busy = false;
  std::atomic<bool> finished{false};
  std::vector<std::shared_ptr<Request>> batch;
  int index_id = 0, k = 0, rows = 0;  // k: the launch's (largest) k
  RerankBounds* h_ks = nullptr;       // the launch's smaller k (FP64 re-check places): pinned
  RerankBounds* d_ks = nullptr;       // and device copies, read by the recorded launch
  std::map<std::tuple<int, int, int>, cudaGraphExec_t> graphs;  // (index, k, class)
  std::map<std::tuple<int, int, int>, bool> no_graph;
};

}  // namespace

struct lshg_server {
  lshg_server_params p{};
  int device = 0;
  std::map<int, Index*> indexes;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::unordered_map<int64_t, std::shared_ptr<Request>> tickets;
  int64_t next_ticket = 1;
  std::vector<std::unique_ptr<Slot>> slots;
  std::map<int, int> busy_slots;  // index id -> slots running it
  std::thread worker;
  bool stop = false;
  int64_t completed = 0, launches = 0, replays = 0, rejected = 0;

  void ensure_buffers(Slot& s, size_t in_elems, size_t out_elems) {
    if (in_elems > s.in_cap) {
      if (s.h_in) cudaFreeHost(s.h_in);
      if (s.d_in) cudaFree(s.d_in);
      LSHG_CUDA(cudaMallocHost((void**)&s.h_in, in_elems * sizeof(float)));
      LSHG_CUDA(cudaMalloc((void**)&s.d_in, in_elems * sizeof(float)));
      s.in_cap = in_elems;
      drop_graphs(s);
    }
    if (out_elems > s.out_cap) {
      if (s.h_out) cudaFreeHost(s.h_out);
      if (s.d_out) cudaFree(s.d_out);
      LSHG_CUDA(cudaMallocHost((void**)&s.h_out, out_elems * sizeof(lshg_point)));
      LSHG_CUDA(cudaMalloc((void**)&s.d_out, out_elems * sizeof(lshg_point)));
      s.out_cap = out_elems;
      drop_graphs(s);
    }
  }

  static void drop_graphs(Slot& s) {
    for (auto& kv : s.graphs) cudaGraphExecDestroy(kv.second);
    s.graphs.clear();
    s.no_graph.clear();
  }

  static void CUDART_CB on_done(void* arg) {
    auto* pr = static_cast<std::pair<lshg_server*, Slot*>*>(arg);
    pr->second->finished.store(true);
    {
      std::lock_guard<std::mutex> g(pr->first->mu);
    }
    pr->first->cv_work.notify_one();
    delete pr;
  }

  // Record the batch into the slot's graph for (index, k, class) or replay it.
  void run_batch(Slot& s, Index& idx, int rows_class) {
    auto key = std::make_tuple(s.index_id, s.k, rows_class);
    if (p.use_graphs && !s.no_graph[key]) {
      auto it = s.graphs.find(key);
      if (it == s.graphs.end()) {
        idx.error_word(s.stream);  // the slot stream's error word exists before the capture
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        bool ok = cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeRelaxed) == cudaSuccess;
        if (ok) {
          try {
            query_index(idx, s.d_in, rows_class, s.k, s.d_out, s.stream, s.d_ks);
          } catch (...) {
            ok = false;
          }
          cudaError_t e = cudaStreamEndCapture(s.stream, &g);
          ok = ok && e == cudaSuccess && g != nullptr;
          if (ok) ok = cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
          if (g) cudaGraphDestroy(g);
        }
        cudaGetLastError();
        if (!ok) {
          s.no_graph[key] = true;
        } else {
          s.graphs[key] = ge;
          it = s.graphs.find(key);
        }
      }
      if (it != s.graphs.end()) {
        LSHG_CUDA(cudaGraphLaunch(it->second, s.stream));
        ++replays;
        return;
      }
    }
    query_index(idx, s.d_in, rows_class, s.k, s.d_out, s.stream, s.d_ks);
  }

  void launch(Slot& s, std::vector<std::shared_ptr<Request>>&& batch) {
    Index& idx = *indexes.at(batch[0]->index_id);
    const int d = idx.d;
    int rows = 0, kmax = 0;
    for (auto& r : batch) {
      rows += r->nq;
      kmax = std::max(kmax, r->k);
    }
    int cls = next_pow2(std::max(1, rows));
    ensure_buffers(s, (size_t)cls * d, (size_t)cls * kmax);
    float* dst = s.h_in;
    for (auto& r : batch) {
      memcpy(dst, r->q.data(), r->q.size() * sizeof(float));
      dst += r->q.size();
    }
    const float* last = s.h_in + (size_t)(rows - 1) * d;
    for (int i = rows; i < cls; ++i) memcpy(s.h_in + (size_t)i * d, last, (size_t)d * sizeof(float));
    s.batch = std::move(batch);
    s.index_id = s.batch[0]->index_id;
    s.k = kmax;
    s.rows = rows;
    std::vector<int> kv;  // distinct k, largest first
    for (auto& r : s.batch)
      if (std::find(kv.begin(), kv.end(), r->k) == kv.end()) kv.push_back(r->k);
    std::sort(kv.begin(), kv.end(), std::greater<int>());
    *s.h_ks = RerankBounds{};
    for (size_t i = 1; i < kv.size() && s.h_ks->n < 4; ++i) s.h_ks->k[s.h_ks->n++] = kv[i];
    s.busy = true;
    s.finished.store(false);
    LSHG_CUDA(cudaMemcpyAsync(s.d_in, s.h_in, (size_t)cls * d * sizeof(float), cudaMemcpyHostToDevice, s.stream));
    LSHG_CUDA(cudaMemcpyAsync(s.d_ks, s.h_ks, sizeof(RerankBounds), cudaMemcpyHostToDevice, s.stream));
    run_batch(s, idx, cls);
    LSHG_CUDA(cudaMemcpyAsync(s.h_out, s.d_out, (size_t)rows * s.k * sizeof(lshg_point), cudaMemcpyDeviceToHost,
                              s.stream));
    LSHG_CUDA(cudaLaunchHostFunc(s.stream, on_done, new std::pair<lshg_server*, Slot*>(this, &s)));
    ++launches;
  }

  void finish(Slot& s) {
    int status = LSHG_OK;
    std::string err;
    try {
      query_error(*indexes.at(s.index_id), s.stream);
    } catch (const Error& e) {
      status = e.status;
      err = e.what();
    }
    cudaError_t ce = cudaStreamSynchronize(s.stream);
    if (ce != cudaSuccess) {
      status = LSHG_ERR_CUDA;
      err = cudaGetErrorString(ce);
    }
    auto now = Clock::now();
    size_t row = 0;
    for (auto& r : s.batch) {  // the first r->k of each of the request's rows
      r->out.resize((size_t)r->nq * r->k);
      for (int i = 0; i < r->nq; ++i, ++row)
        memcpy(r->out.data() + (size_t)i * r->k, s.h_out + row * s.k, (size_t)r->k * sizeof(lshg_point));
      r->t_done = now;
      r->status = status;
      r->err = err;
      r->state = status == LSHG_OK ? 2 : 3;
      ++completed;
    }
    s.batch.clear();
    s.busy = false;
  }

  // Next batch for a free slot, or empty (then *wait_us is how long until the oldest
  // eligible request's batching window closes, or -1).  Called with mu held.
  std::vector<std::shared_ptr<Request>> take_batch(Clock::time_point now, int64_t* wait_us) {
    *wait_us = -1;
    // an index keeps one slot free for the others while requests for another index wait
    bool mixed = false;
    for (auto& r : queue)
      if (r->index_id != queue.front()->index_id) {
        mixed = true;
        break;
      }
    const int cap = (mixed && slots.size() > 1) ? (int)slots.size() - 1 : (int)slots.size();
    std::shared_ptr<Request> first;
    for (auto& r : queue)
      if (busy_slots[r->index_id] < cap) {
        first = r;
        break;
      }
    if (!first) return {};
    const Index& I = *indexes.at(first->index_id);
    const int cls = batch_class(I, first->k);
    auto same = [&](const Request& r) {
      return r.index_id == first->index_id && batch_class(*indexes.at(r.index_id), r.k) == cls;
    };
    int avail = 0;
    for (auto& r : queue)
      if (same(*r)) avail += r->nq;
    const int64_t age = std::chrono::duration_cast<std::chrono::microseconds>(now - first->t_submit).count();
    if (p.batch_window_us > 0 && avail < p.max_batch && age < p.batch_window_us) {
      *wait_us = p.batch_window_us - age;
      return {};
    }
    std::vector<std::shared_ptr<Request>> batch;
    std::vector<int> kv;  // at most four distinct k a launch
    int rows = 0;
    for (auto it = queue.begin(); it != queue.end();) {
      auto& r = *it;
      const bool newk = std::find(kv.begin(), kv.end(), r->k) == kv.end();
      if (same(*r) && rows + r->nq <= p.max_batch && (!newk || kv.size() < 4)) {
        if (newk) kv.push_back(r->k);
        rows += r->nq;
        r->state = 1;
        batch.push_back(r);
        it = queue.erase(it);
      } else {
        ++it;
      }
    }
    return batch;
  }

  void loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      bool progressed = false;
      for (auto& sp : slots) {
        Slot& s = *sp;
        if (s.busy && s.finished.load()) {
          const int iid = s.index_id;
          lk.unlock();
          finish(s);
          lk.lock();
          --busy_slots[iid];
          progressed = true;
          cv_done.notify_all();
        }
      }
      int64_t wait_us = -1;
      for (auto& sp : slots) {
        Slot& s = *sp;
        if (s.busy || queue.empty()) continue;
        int64_t w = -1;
        auto batch = take_batch(Clock::now(), &w);
        if (batch.empty()) {
          if (w >= 0 && (wait_us < 0 || w < wait_us)) wait_us = w;
          continue;
        }
        const int iid = batch[0]->index_id;
        ++busy_slots[iid];
        lk.unlock();
        try {
          launch(s, std::move(batch));
        } catch (const Error& e) {
          for (auto& r : s.batch.empty() ? batch : s.batch) {
            r->status = e.status;
            r->err = e.what();
            r->state = 3;
          }
          s.batch.clear();
          s.busy = false;
          cudaGetLastError();
        }
        lk.lock();
        if (!s.busy) --busy_slots[iid];
        progressed = true;
        cv_done.notify_all();
      }
      if (stop) {
        bool any = false;
        for (auto& sp : slots) any = any || sp->busy;
        if (!any) break;
      }
      if (!progressed)
        cv_work.wait_for(lk, std::chrono::microseconds(wait_us >= 0 ? std::max<int64_t>(1, std::min<int64_t>(wait_us, 200))
                                                                    : 200));
    }
  }
};

extern "C" {

void lshg_server_params_default(lshg_server_params* p) {
  if (!p) return;
  p->max_batch = 4096;
  p->max_queue = 65536;
  p->streams = 2;
  p->use_graphs = 1;
  p->hbm_reserve_mb = 1024;
  p->batch_window_us = 0;
}

int lshg_server_create(const lshg_server_params* p, lshg_server** out) {
  if (!p || !out) return LSHG_ERR_INVALID_ARGUMENT;
  try {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return LSHG_ERR_NO_DEVICE;
    auto* s = new lshg_server();
    s->p = *p;
    if (s->p.max_batch < 1) s->p.max_batch = 4096;
    if (s->p.streams < 1) s->p.streams = 1;
    cudaGetDevice(&s->device);
    for (int i = 0; i < s->p.streams; ++i) {
      auto sl = std::make_unique<Slot>();
      LSHG_CUDA(cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking));
      LSHG_CUDA(cudaMallocHost((void**)&sl->h_ks, sizeof(RerankBounds)));
      LSHG_CUDA(cudaMalloc((void**)&sl->d_ks, sizeof(RerankBounds)));
      *sl->h_ks = RerankBounds{};
      s->slots.push_back(std::move(sl));
    }
    s->worker = std::thread([s] { s->loop(); });
    *out = s;
    return LSHG_OK;
  } catch (const Error& e) {
    return e.status;
  }
}

int lshg_server_add_index(lshg_server* s, int index_id, lshg_index* idx) {
  if (!s || !idx || !idx->impl) return LSHG_ERR_INVALID_ARGUMENT;
  if (idx->impl->device != s->device) {
    set_last_error("the index lives on another device than the server");
    return LSHG_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(s->mu);
  s->indexes[index_id] = idx->impl.get();
  return LSHG_OK;
}

int lshg_server_submit(lshg_server* s, int index_id, const float* queries, int N_query, int k, int64_t* ticket) {
  if (!s || !queries || !ticket || N_query < 1 || k < 1 || k > 4096) return LSHG_ERR_INVALID_ARGUMENT;
  Index* idx;
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->indexes.find(index_id);
    if (it == s->indexes.end()) return LSHG_ERR_INVALID_ARGUMENT;
    idx = it->second;
    if (N_query > s->p.max_batch) return LSHG_ERR_INVALID_ARGUMENT;
    if ((int)s->queue.size() >= s->p.max_queue) {
      ++s->rejected;
      return LSHG_ERR_BUSY;
    }
  }
  // admission by free HBM: the request's buffers plus scratch must fit above the reserve
  size_t free_b = 0, total_b = 0;
  cudaSetDevice(s->device);
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
    int64_t need = (int64_t)N_query * (idx->d * 4 + k * 8) * 4 + (int64_t)N_query * 4096 * 8;
    if ((int64_t)free_b - need < s->p.hbm_reserve_mb * (int64_t)(1 << 20)) {
      std::lock_guard<std::mutex> g(s->mu);
      ++s->rejected;
      return LSHG_ERR_BUSY;
    }
  }
  auto r = std::make_shared<Request>();
  r->index_id = index_id;
  r->nq = N_query;
  r->k = k;
  r->q.assign(queries, queries + (size_t)N_query * idx->d);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->ticket = s->next_ticket++;
    s->tickets[r->ticket] = r;
    s->queue.push_back(r);
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  return LSHG_OK;
}

int lshg_server_wait(lshg_server* s, int64_t ticket, lshg_point* results, int64_t timeout_us, double* latency_us) {
  if (!s || !results) return LSHG_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return LSHG_ERR_INVALID_ARGUMENT;
  auto r = it->second;
  bool ok = s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return r->state >= 2; });
  if (!ok) return LSHG_ERR_TIMEOUT;
  s->tickets.erase(ticket);
  if (r->state == 3) return r->status;
  memcpy(results, r->out.data(), r->out.size() * sizeof(lshg_point));
  if (latency_us) *latency_us = std::chrono::duration<double, std::micro>(r->t_done - r->t_submit).count();
  return LSHG_OK;
}

int lshg_server_stats(lshg_server* s, int64_t* completed, int64_t* launches, int64_t* graph_replays,
                      int64_t* rejected) {
  if (!s) return LSHG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  if (completed) *completed = s->completed;
  if (launches) *launches = s->launches;
  if (graph_replays) *graph_replays = s->replays;
  if (rejected) *rejected = s->rejected;
  return LSHG_OK;
}

int lshg_server_destroy(lshg_server* s) {
  if (!s) return LSHG_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto& sl : s->slots) {
    cudaStreamSynchronize(sl->stream);
    lshg_server::drop_graphs(*sl);
    if (sl->h_in) cudaFreeHost(sl->h_in);
    if (sl->d_in) cudaFree(sl->d_in);
    if (sl->h_out) cudaFreeHost(sl->h_out);
    if (sl->d_out) cudaFree(sl->d_out);
    if (sl->h_ks) cudaFreeHost(sl->h_ks);
    if (sl->d_ks) cudaFree(sl->d_ks);
    cudaStreamDestroy(sl->stream);
  }
  delete s;
  return LSHG_OK;
}

}  // extern "C"
