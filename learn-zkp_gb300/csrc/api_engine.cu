// libbasefold_gpu.so: the prover engine — many commit+eval+open jobs of
// different sizes in flight at once (batched and served forms).
//
// Each job follows the reference's harness (poly-commit/src/lib.rs:80-100):
// commit, observe the root, evaluate at the point, observe the value, open
// with a fresh keccak256 transcript.  A job runs on one stream of a pool.  At
// admission the whole commit, evaluation and open up to the final polynomial
// are enqueued at once, with the transcript on the device, so the GPU never
// waits for the host inside a proof; the host then samples the query
// positions from the returned transcript and reads the openings.  The engine
// admits jobs while streams and the HBM budget allow and advances whichever
// job's GPU work has finished, so small latency-bound proofs overlap with
// large ones and new requests join while others run (continuous batching).
// Proof bytes are identical to the one-at-a-time path.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "api_common.h"

using bfh::u128;
using namespace bfapi;

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// J_OPEN: GPU work up to the final polynomial in flight; J_COMPLETING: a
// completion thread samples the queries, gathers the openings and writes the
// proof; J_DONE: retired.
enum JobState { J_OPEN = 0, J_COMPLETING = 1, J_DONE = 2 };

// One size's job captured on one slot: fixed buffers (evaluations,
// codeword, trees, open workspace) and the CUDA graph that runs commit,
// evaluation and the device-transcript open on them.  A job of that size on
// that slot writes its point into the staging, copies its evaluations in and
// replays the graph.
struct Plan {
  int n = -1;
  bf_pcs* p = nullptr;
  std::unique_ptr<bf_commitment> cm;
  DevBuf eval_ws;
  bf_open_session* sess = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long launches = 0;  // kernels per replay
  size_t footprint = 0;
  uint64_t last_use = 0;   // admission counter value of its last job (LRU eviction)
  ~Plan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (sess) bf_open_session_free(sess);
  }
};

struct Job {
  bf_job* pub = nullptr;
  Plan* plan = nullptr;  // graph replay: the session and buffers belong to the plan
  bool device_input = false;
  double t_submit = 0;
  bf_pcs* pcs = nullptr;
  int slot = -1;
  cudaStream_t st = nullptr;
  std::unique_ptr<bf_commitment> cm;
  bf_open_session* sess = nullptr;
  bfh::Challenger ch;
  DevBuf eval_ws;
  int state = J_OPEN;
  size_t footprint = 0;
  std::atomic<bool> completed{false};  // set by the completion thread
  int complete_rc = 0;
};

}  // namespace

struct bf_engine {
  int device = 0, lambda = 128, log2_c = 1, max_inflight = 8;
  int autotune_reps = 0;  // > 0: autotune each size's pcs when it is created
  bool has_tune = false;  // launch shapes set for every size (bf_engine_set_tune)
  int tune_vals[bf::kTuneVals] = {};
  int tune_n = 4;
  bool use_graphs = false;  // replay one captured graph per (slot, size)
  std::vector<std::map<int, std::unique_ptr<Plan>>> plans;  // per slot, by size
  uint64_t admissions = 0;
  // host-side accounting (bf_engine_stats)
  double host_ms_enqueue = 0, host_ms_launch = 0, host_ms_complete = 0;
  uint64_t plans_built = 0, plans_dropped = 0, jobs_done = 0;
  // Completion threads: query sampling, gather and proof readout of jobs
  // whose GPU work is done, off the scheduling thread.
  std::vector<std::thread> completers;
  std::deque<Job*> complete_q;
  std::mutex complete_mu;
  std::condition_variable complete_cv;
  bool complete_stop = false;
  size_t mem_budget = 0, mem_used = 0;
  std::map<int, bf_pcs*> pcs_by_n;
  std::mutex pcs_mu;  // pcs_by_n: bf_engine_proof_size may set a size up while the engine runs
  std::vector<cudaStream_t> streams;
  // Per slot, a stream of the device's highest priority: jobs of at most
  // prio_max_vars variables run there, so their blocks are dispatched ahead
  // of waiting blocks of larger jobs (whose long kernels retire blocks
  // continuously).  -1: off.
  std::vector<cudaStream_t> streams_hi;
  int prio_max_vars = -1;
  bool smallest_first = false;  // admit the smallest queued job first (else in arrival order)
  std::vector<int> free_slots;
  PinnedBuf pin;  // 128 bytes per slot: roots (64) + value (16)
  std::deque<Job*> queue;
  std::vector<Job*> inflight;
  std::vector<bf_job*> finished;  // completed, not yet collected by bf_engine_poll
  std::mutex mu;
  std::condition_variable cv;
  std::thread worker;
  bool running = false;
  bool stop = false;
  size_t outstanding = 0;  // submitted and not finished
  ~bf_engine();
};

namespace {

size_t job_footprint(int n, int log2_c, bool device_input, size_t Q, size_t block_bytes) {
  const size_t N = (size_t)1 << n, c = (size_t)1 << log2_c;
  size_t b = (40 + 160 * c) * N + Q * block_bytes + (2u << 20);
  if (!device_input) b += 16 * N;
  return b;
}

int get_pcs(bf_engine* e, int n, bf_pcs** out) {
  std::lock_guard<std::mutex> lk(e->pcs_mu);
  auto it = e->pcs_by_n.find(n);
  if (it != e->pcs_by_n.end()) {
    *out = it->second;
    return BF_OK;
  }
  bf_pcs* p = nullptr;
  // its own stream: a slot's stream may be in graph capture meanwhile
  TRY(bf_pcs_setup(e->device, e->lambda, e->log2_c, n, nullptr, &p));
  e->pcs_by_n[n] = p;
  if (e->has_tune) TRY(bf_pcs_set_tune(p, e->tune_vals, e->tune_n));
  if (e->autotune_reps > 0) TRY(bf_pcs_autotune(p, e->autotune_reps, nullptr, 0));
  *out = p;
  return BF_OK;
}

void finish_job(bf_engine* e, Job* j, int status) {
  j->pub->status = status;
  j->pub->latency_ms = now_ms() - j->t_submit;
  if (j->plan) {
    if (status < 0 && j->slot >= 0) {  // a failed job may leave the plan mid-way: rebuild it next time
      auto& m = e->plans[j->slot];
      auto it = m.find(j->plan->n);
      if (it != m.end()) {
        e->mem_used -= it->second->footprint;
        m.erase(it);
      }
    }
    j->sess = nullptr;
    j->plan = nullptr;
  }
  if (j->sess) {
    bf_open_session_free(j->sess);
    j->sess = nullptr;
  }
  j->eval_ws.release();
  j->cm.reset();
  if (j->slot >= 0) e->free_slots.push_back(j->slot);
  e->mem_used -= j->footprint;
  e->jobs_done += 1;
  j->state = J_DONE;
}

uint8_t* slot_pin(bf_engine* e, int slot) { return e->pin.b() + 128 * (size_t)slot; }

// Starts a job on a free slot: allocate, copy the evaluations in, enqueue
// the commit, the evaluation and the device-transcript open.
int admit(bf_engine* e, Job* j) {
  bf_job* pj = j->pub;
  TRY(get_pcs(e, pj->num_vars, &j->pcs));
  bf_pcs* p = j->pcs;
  const size_t need = bf_pcs_proof_size(p, 1, 1);
  if (pj->proof_cap < need) return fail(BF_ERR_BUFFER, "job proof buffer needs %zu bytes", need);
  const bool hi = e->prio_max_vars >= 0 && pj->num_vars <= e->prio_max_vars && !e->streams_hi.empty();
  j->st = hi ? e->streams_hi[j->slot] : e->streams[j->slot];
  j->cm.reset(new bf_commitment());
  j->cm->pcs = p;
  j->cm->width = 1;
  const size_t bytes = 16 * ((size_t)1 << p->d);
  if (j->device_input) {
    if (reinterpret_cast<uintptr_t>(pj->evals) & 15) return fail(BF_ERR_ARG, "device evaluations must be 16-byte aligned");
    j->cm->data.p = const_cast<void*>(pj->evals);
    j->cm->data.owned = false;
    j->cm->data.bytes = bytes;
  } else {
    CU(j->cm->data.alloc_async(bytes, p->pool, j->st));
    CU(cudaMemcpyAsync(j->cm->data.p, pj->evals, bytes, cudaMemcpyHostToDevice, j->st));
  }
  uint8_t* pin = slot_pin(e, j->slot);
  TRY(commit_enqueue(p, j->cm.get(), j->cm->data.as<uint4>(), j->st, pin));
  const size_t half = p->d > 0 ? ((size_t)1 << (p->d - 1)) : 1;
  CU(j->eval_ws.alloc_async(16 * half, p->pool, j->st));
  const uint4* value_dev = nullptr;
  TRY(eval_enqueue(p, j->cm.get(), pj->point, j->eval_ws.as<uint4>(), j->st, pin + 64, &value_dev));
  TRY(open_start_impl(p, j->cm.get(), pj->point, nullptr, nullptr, j->st, &j->sess));
  const size_t nd = p->n_d();
  const uint4* root_dev = j->cm->tree.as<uint4>() + 2 * (2 * nd - 2);
  j->ch = bfh::Challenger();  // GenericChallenger::keccak256()
  TRY(open_resident_enqueue(j->sess, j->ch, root_dev, value_dev));
  j->state = J_OPEN;
  return BF_OK;
}

// Enqueues one job's GPU work on the plan's buffers (captured once).
int capture_job(bf_engine* e, int slot, Plan* pl) {
  bf_pcs* p = pl->p;
  bf_commitment* cm = pl->cm.get();
  cudaStream_t st = e->streams[slot];
  uint8_t* pin = slot_pin(e, slot);
  TRY(open_session_enqueue_start(pl->sess));  // copies the point first: the evaluation reads it
  TRY(commit_enqueue(p, cm, cm->data.as<uint4>(), st, pin));
  const uint4* value_dev = nullptr;
  TRY(eval_enqueue(p, cm, nullptr, pl->eval_ws.as<uint4>(), st, pin + 64, &value_dev,
                   open_session_point_dev(pl->sess)));
  const uint4* root_dev = cm->tree.as<uint4>() + 2 * (2 * p->n_d() - 2);
  TRY(open_resident_enqueue_device(pl->sess, root_dev, value_dev));
  return BF_OK;
}

int build_plan(bf_engine* e, int slot, int n, std::unique_ptr<Plan>& out) {
  std::unique_ptr<Plan> pl(new Plan());
  pl->n = n;
  TRY(get_pcs(e, n, &pl->p));
  bf_pcs* p = pl->p;
  cudaStream_t st = e->streams[slot];
  pl->cm.reset(new bf_commitment());
  pl->cm->pcs = p;
  pl->cm->width = 1;
  CU(pl->cm->data.alloc_async(16 * ((size_t)1 << n), p->pool, st));
  TRY(commit_alloc(p, pl->cm.get(), st));
  CU(pl->eval_ws.alloc_async(16 * (n > 0 ? ((size_t)1 << (n - 1)) : 1), p->pool, st));
  TRY(open_session_create(p, pl->cm.get(), st, &pl->sess));
  const long long before = (long long)bf::launches_this_thread();  // completions launch meanwhile
  cudaGraph_t graph = nullptr;
  CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int rc = capture_job(e, slot, pl.get());
  const cudaError_t ce = cudaStreamEndCapture(st, &graph);
  pl->launches = (long long)bf::launches_this_thread() - before;
  bf::add_launches(-pl->launches);  // captured, not run
  if (rc < 0) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  CU(ce);
  const cudaError_t ie = cudaGraphInstantiate(&pl->exec, graph, 0);
  cudaGraphDestroy(graph);
  CU(ie);
  const size_t Q = p->Q;
  pl->footprint = job_footprint(n, e->log2_c, false, Q, p->block_bytes(1));
  out = std::move(pl);
  return BF_OK;
}

// Graph replay of a job on its slot's plan for its size (built by progress()).
int admit_graph(bf_engine* e, Job* j) {
  bf_job* pj = j->pub;
  Plan* pl = e->plans[j->slot][pj->num_vars].get();
  pl->last_use = ++e->admissions;
  j->plan = pl;
  j->pcs = pl->p;
  j->st = e->streams[j->slot];
  j->sess = pl->sess;
  const size_t need = bf_pcs_proof_size(pl->p, 1, 1);
  if (pj->proof_cap < need) return fail(BF_ERR_BUFFER, "job proof buffer needs %zu bytes", need);
  if (j->device_input && (reinterpret_cast<uintptr_t>(pj->evals) & 15))
    return fail(BF_ERR_ARG, "device evaluations must be 16-byte aligned");
  TRY(open_session_prepare(pl->sess, pj->point, nullptr, nullptr));
  j->ch = bfh::Challenger();  // GenericChallenger::keccak256()
  TRY(open_resident_prepare(pl->sess, j->ch));
  CU(cudaMemcpyAsync(pl->cm->data.p, pj->evals, 16 * ((size_t)1 << pl->n),
                     j->device_input ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, j->st));
  const double t0 = now_ms();
  CU(cudaGraphLaunch(pl->exec, j->st));
  e->host_ms_launch += now_ms() - t0;
  bf::add_launches(pl->launches);
  CU(cudaEventRecord(open_session_event(pl->sess), j->st));
  open_session_mark_launched(pl->sess);
  j->state = J_OPEN;
  return BF_OK;
}

// The completion of one job (on a completion thread): read the rounds and
// the transcript, sample the query positions (basefold.rs:200-203), gather
// the openings and write the proof, root and value.
int complete_job(bf_engine* e, Job* j) {
  bf_pcs* p = j->pcs;
  bf_job* pj = j->pub;
  TRY(open_resident_complete(j->sess, j->ch));
  std::vector<uint64_t> idx(p->Q);
  for (size_t q = 0; q < p->Q; ++q) idx[q] = j->ch.sample_bits(p->L);
  // The gather and proof readout go to the slot's high-priority stream: the
  // job's rounds are done, and its blocks then start ahead of the waiting
  // blocks of other jobs' long kernels instead of behind them, so the slot
  // (and its memory) is released sooner.
  const cudaStream_t own = open_session_stream(j->sess);
  const cudaStream_t fast = e->streams_hi.empty() ? own : e->streams_hi[j->slot];
  open_session_set_stream(j->sess, fast);
  int rc = open_finish_enqueue(j->sess, idx.data(), idx.size());
  if (rc >= 0) rc = open_finish_complete(j->sess, pj->proof, pj->proof_cap, &pj->proof_len);
  open_session_set_stream(j->sess, own);
  TRY(rc);
  bfh::digest_from_interleaved(slot_pin(e, j->slot), pj->root);  // the tree root, stored interleaved
  std::memcpy(pj->value, slot_pin(e, j->slot) + 64, 16);
  return BF_OK;
}

void completer_loop(bf_engine* e) {
  cudaSetDevice(e->device);
  while (true) {
    Job* j = nullptr;
    {
      std::unique_lock<std::mutex> lk(e->complete_mu);
      e->complete_cv.wait(lk, [e] { return e->complete_stop || !e->complete_q.empty(); });
      if (e->complete_q.empty()) return;  // stopping and drained
      j = e->complete_q.front();
      e->complete_q.pop_front();
    }
    const double t0 = now_ms();
    j->complete_rc = complete_job(e, j);
    const double dt = now_ms() - t0;
    {
      std::lock_guard<std::mutex> lk(e->complete_mu);
      e->host_ms_complete += dt;
    }
    j->completed.store(true, std::memory_order_release);
  }
}

// Advances a job whose GPU work has completed.  Returns 1 if it moved.
int step(bf_engine* e, Job* j) {
  if (j->state == J_OPEN) {
    int ready = bf_open_poll(j->sess);
    TRY(ready);
    if (!ready) return 0;
    j->state = J_COMPLETING;
    {
      std::lock_guard<std::mutex> lk(e->complete_mu);
      e->complete_q.push_back(j);
    }
    e->complete_cv.notify_one();
    return 1;
  }
  if (j->state == J_COMPLETING) {
    if (!j->completed.load(std::memory_order_acquire)) return 0;
    TRY(j->complete_rc);
    finish_job(e, j, BF_OK);
    return 1;
  }
  return 0;
}

// One pass over the engine: admit what fits, advance what is ready, retire
// finished jobs.  Called with e->mu held only around queue access.
bool progress(bf_engine* e) {
  bool moved = false;
  while (true) {
    Job* j = nullptr;
    int slot = -1;
    {
      std::lock_guard<std::mutex> lk(e->mu);
      if (e->queue.empty() || e->free_slots.empty()) break;
      auto qit = e->queue.begin();
      if (e->smallest_first)
        for (auto it = e->queue.begin(); it != e->queue.end(); ++it)
          if ((*it)->pub->num_vars < (*qit)->pub->num_vars) qit = it;
      Job* cand = *qit;
      if (e->use_graphs) {
        // a free slot that has a plan of this size, else the free slot with the
        // least plan memory; room for a new plan comes from idle plans, least
        // recently used first (always admit when idle so oversized jobs run)
        const int n = cand->pub->num_vars;
        size_t pick = e->free_slots.size();
        for (size_t k = 0; k < e->free_slots.size() && pick == e->free_slots.size(); ++k)
          if (e->plans[e->free_slots[k]].count(n)) pick = k;
        if (pick == e->free_slots.size()) {
          size_t best = ~(size_t)0;
          for (size_t k = 0; k < e->free_slots.size(); ++k) {
            size_t held = 0;
            for (auto& kv : e->plans[e->free_slots[k]]) held += kv.second->footprint;
            if (held < best) {
              best = held;
              pick = k;
            }
          }
          while (e->mem_used + cand->footprint > e->mem_budget) {
            Plan* victim = nullptr;
            int vslot = -1;
            for (int fs : e->free_slots)
              for (auto& kv : e->plans[fs])
                if (!victim || kv.second->last_use < victim->last_use) {
                  victim = kv.second.get();
                  vslot = fs;
                }
            if (!victim) break;
            e->mem_used -= victim->footprint;
            e->plans[vslot].erase(victim->n);
            e->plans_dropped += 1;
          }
          if (!e->inflight.empty() && e->mem_used + cand->footprint > e->mem_budget) break;
        }
        slot = e->free_slots[pick];
        e->free_slots.erase(e->free_slots.begin() + pick);
      } else {
        // admission by HBM footprint: always admit when idle so oversized jobs still run
        if (!e->inflight.empty() && e->mem_used + cand->footprint > e->mem_budget) break;
        slot = e->free_slots.back();
        e->free_slots.pop_back();
      }
      e->queue.erase(qit);
      j = cand;
    }
    j->slot = slot;
    e->inflight.push_back(j);
    int rc = BF_OK;
    const double t_enq = now_ms();
    if (e->use_graphs) {
      j->footprint = 0;  // memory is held by the slot's plan
      const int n = j->pub->num_vars;
      if (!e->plans[slot].count(n)) {
        std::unique_ptr<Plan> pl;
        rc = build_plan(e, slot, n, pl);
        if (rc >= 0) {
          e->mem_used += pl->footprint;
          e->plans[slot][n] = std::move(pl);
          e->plans_built += 1;
        }
      }
      if (rc >= 0) rc = admit_graph(e, j);
    } else {
      e->mem_used += j->footprint;
      rc = admit(e, j);
    }
    e->host_ms_enqueue += now_ms() - t_enq;
    if (rc < 0) finish_job(e, j, rc);
    moved = true;
  }
  for (Job* j : e->inflight) {
    if (j->state == J_DONE) continue;
    int rc = step(e, j);
    if (rc < 0) finish_job(e, j, rc);
    if (rc != 0) moved = true;
  }
  std::vector<Job*> keep;
  for (Job* j : e->inflight) {
    if (j->state == J_DONE) {
      std::lock_guard<std::mutex> lk(e->mu);
      e->finished.push_back(j->pub);
      e->outstanding -= 1;
      delete j;
      e->cv.notify_all();
    } else {
      keep.push_back(j);
    }
  }
  e->inflight.swap(keep);
  return moved;
}

void worker_loop(bf_engine* e) {
  cudaSetDevice(e->device);
  while (true) {
    {
      std::unique_lock<std::mutex> lk(e->mu);
      if (e->stop && e->outstanding == 0) break;
      if (e->outstanding == 0) {
        e->cv.wait_for(lk, std::chrono::milliseconds(5));
        continue;
      }
    }
    if (!progress(e)) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

}  // namespace

bf_engine::~bf_engine() {
  for (cudaStream_t s : streams) cudaStreamSynchronize(s);
  for (cudaStream_t s : streams_hi) cudaStreamSynchronize(s);
  plans.clear();
  for (auto& kv : pcs_by_n) bf_pcs_free(kv.second);
  for (cudaStream_t s : streams) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  for (cudaStream_t s : streams_hi) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
}

extern "C" {

int bf_engine_create(int device, int lambda, int log2_c, int max_inflight, size_t mem_budget, bf_engine** out) {
  if (!out || max_inflight <= 0 || max_inflight > 256 || log2_c < 0 || log2_c > 4)
    return fail(BF_ERR_ARG, "bad engine parameters");
  *out = nullptr;
  CU(cudaSetDevice(device));
  std::unique_ptr<bf_engine> e(new bf_engine());
  e->device = device;
  e->lambda = lambda;
  e->log2_c = log2_c;
  e->max_inflight = max_inflight;
  if (mem_budget == 0) {
    size_t free_b = 0, total_b = 0;
    CU(cudaMemGetInfo(&free_b, &total_b));
    mem_budget = free_b / 10 * 8;
  }
  e->mem_budget = mem_budget;
  int prio_least = 0, prio_greatest = 0;
  CU(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
  for (int i = 0; i < max_inflight; ++i) {
    cudaStream_t s;
    CU(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    e->streams.push_back(s);
    e->free_slots.push_back(max_inflight - 1 - i);
    if (prio_greatest != prio_least) {
      CU(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio_greatest));
      e->streams_hi.push_back(s);
    }
  }
  CU(e->pin.ensure(128 * (size_t)max_inflight));
  e->plans.resize(max_inflight);
  // Completion threads mostly wait for a job's gather and proof readout, so
  // there is one per two slots (at least one, at most 16) rather than per core.
  const int n_completers = std::max(1, std::min(16, max_inflight / 2));
  for (int i = 0; i < n_completers; ++i) e->completers.emplace_back(completer_loop, e.get());
  *out = e.release();
  return BF_OK;
}

void bf_engine_free(bf_engine* e) {
  if (!e) return;
  if (e->running) {
    {
      std::lock_guard<std::mutex> lk(e->mu);
      e->stop = true;
      e->cv.notify_all();
    }
    e->worker.join();
  }
  // jobs with a completion thread are left to finish it first
  for (Job* j : e->inflight)
    while (j->state == J_COMPLETING && !j->completed.load(std::memory_order_acquire))
      std::this_thread::sleep_for(std::chrono::microseconds(50));
  {
    std::lock_guard<std::mutex> lk(e->complete_mu);
    e->complete_stop = true;
  }
  e->complete_cv.notify_all();
  for (auto& t : e->completers) t.join();
  for (Job* j : e->inflight) {
    finish_job(e, j, BF_ERR_ARG);
    delete j;
  }
  for (Job* j : e->queue) delete j;
  DeviceGuard g(e->device);
  delete e;
}

size_t bf_engine_proof_size(bf_engine* e, int num_vars) {
  if (!e || num_vars < 0) return 0;
  bf_pcs* p = nullptr;
  if (get_pcs(e, num_vars, &p) < 0) return 0;
  return bf_pcs_proof_size(p, 1, 1);
}

int bf_engine_submit(bf_engine* e, bf_job* job, int device_input) {
  if (!e || !job || !job->evals || (job->num_vars > 0 && !job->point) || !job->proof)
    return fail(BF_ERR_ARG, "null argument");
  if (job->num_vars < 0 || job->num_vars + e->log2_c > 30) return fail(BF_ERR_ARG, "bad num_vars");
  Job* j = new Job();
  j->pub = job;
  j->device_input = device_input != 0;
  j->t_submit = now_ms();
  job->status = 1;  // pending
  job->proof_len = 0;
  const size_t Q = num_queries(e->lambda, e->log2_c);
  size_t bb = 8 + 16 + 8 + 32 * (size_t)(job->num_vars + e->log2_c) + 8;
  for (int i = 0; i < job->num_vars; ++i) bb += 24 + 32 * (size_t)(e->log2_c + i);
  j->footprint = job_footprint(job->num_vars, e->log2_c, j->device_input, Q, bb);
  std::lock_guard<std::mutex> lk(e->mu);
  e->queue.push_back(j);
  e->outstanding += 1;
  e->cv.notify_all();
  return BF_OK;
}

int bf_engine_cancel(bf_engine* e, bf_job* job) {
  if (!e || !job) return fail(BF_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(e->mu);
  for (auto it = e->queue.begin(); it != e->queue.end(); ++it) {
    Job* j = *it;
    if (j->pub != job) continue;
    e->queue.erase(it);
    job->status = BF_ERR_CANCELLED;
    job->latency_ms = now_ms() - j->t_submit;
    delete j;
    e->finished.push_back(job);  // returned by bf_engine_poll like any finished job
    e->outstanding -= 1;
    e->cv.notify_all();
    return BF_OK;
  }
  return fail(BF_ERR_ARG, "job is not waiting for admission (already running or finished)");
}

int bf_engine_stats(bf_engine* e, double* out, int n) {
  if (!e || !out || n < 6) return fail(BF_ERR_ARG, "need 6 values");
  std::lock_guard<std::mutex> lk(e->mu);
  out[0] = e->host_ms_enqueue;
  out[1] = e->host_ms_launch;
  {
    std::lock_guard<std::mutex> lk2(e->complete_mu);
    out[2] = e->host_ms_complete;
  }
  out[3] = (double)e->plans_built;
  out[4] = (double)e->plans_dropped;
  out[5] = (double)e->jobs_done;
  return BF_OK;
}

int bf_engine_graphs(bf_engine* e, int on) {
  if (!e) return fail(BF_ERR_ARG, "null argument");
  if (e->running || !e->inflight.empty()) return fail(BF_ERR_ARG, "engine busy");
  e->use_graphs = on != 0;
  if (!e->use_graphs) {
    for (auto& m : e->plans) {
      for (auto& kv : m) e->mem_used -= kv.second->footprint;
      m.clear();
    }
  }
  return BF_OK;
}

int bf_engine_set_tune(bf_engine* e, const int* vals, int n) {
  if (!e || !vals || n < 4) return fail(BF_ERR_ARG, "need at least 4 values");
  if (e->running || !e->inflight.empty()) return fail(BF_ERR_ARG, "engine busy");
  std::lock_guard<std::mutex> lk(e->pcs_mu);
  for (auto& kv : e->pcs_by_n) TRY(bf_pcs_set_tune(kv.second, vals, n));
  if (e->pcs_by_n.empty()) {  // validate now: a later setup would fail on it
    bf_pcs* probe = nullptr;
    TRY(bf_pcs_setup(-1, e->lambda, e->log2_c, 1, nullptr, &probe));
    const int rc = bf_pcs_set_tune(probe, vals, n);
    bf_pcs_free(probe);
    TRY(rc);
  }
  e->tune_n = n < bf::kTuneVals ? n : bf::kTuneVals;
  std::memcpy(e->tune_vals, vals, sizeof(int) * (size_t)e->tune_n);
  e->has_tune = true;
  return BF_OK;
}

int bf_engine_schedule(bf_engine* e, int smallest_first, int prio_max_vars) {
  if (!e || prio_max_vars < -1 || prio_max_vars > 30) return fail(BF_ERR_ARG, "bad argument");
  if (e->running || !e->inflight.empty()) return fail(BF_ERR_ARG, "engine busy");
  e->smallest_first = smallest_first != 0;
  e->prio_max_vars = prio_max_vars;
  return BF_OK;
}

int bf_engine_autotune(bf_engine* e, int reps) {
  if (!e || reps < 0 || reps > 100) return fail(BF_ERR_ARG, "bad argument");
  e->autotune_reps = reps;
  return BF_OK;
}

int bf_engine_start(bf_engine* e) {
  if (!e) return fail(BF_ERR_ARG, "null argument");
  if (e->running) return BF_OK;
  e->stop = false;
  e->running = true;
  e->worker = std::thread(worker_loop, e);
  return BF_OK;
}

int bf_engine_stop(bf_engine* e) {
  if (!e) return fail(BF_ERR_ARG, "null argument");
  if (!e->running) return BF_OK;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    e->stop = true;
    e->cv.notify_all();
  }
  e->worker.join();
  e->running = false;
  return BF_OK;
}

int bf_engine_poll(bf_engine* e, bf_job** done, size_t cap, size_t* n) {
  if (!e || !n) return fail(BF_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(e->mu);
  size_t k = 0;
  while (k < cap && !e->finished.empty()) {
    if (done) done[k] = e->finished.front();
    e->finished.erase(e->finished.begin());
    ++k;
  }
  *n = k;
  return BF_OK;
}

int bf_engine_prove(bf_engine* e, bf_job* jobs, size_t count, int device_input) {
  if (!e || (count && !jobs)) return fail(BF_ERR_ARG, "null argument");
  if (e->running) return fail(BF_ERR_ARG, "engine is serving; use bf_engine_submit");
  DeviceGuard g(e->device);
  for (size_t i = 0; i < count; ++i) TRY(bf_engine_submit(e, &jobs[i], device_input));
  while (true) {
    {
      std::lock_guard<std::mutex> lk(e->mu);
      if (e->outstanding == 0) break;
    }
    if (!progress(e)) std::this_thread::yield();
  }
  std::lock_guard<std::mutex> lk(e->mu);
  e->finished.clear();
  for (size_t i = 0; i < count; ++i)
    if (jobs[i].status < 0) return jobs[i].status;
  return BF_OK;
}

}  // extern "C"
