// Serving path: resident form-factor rows, continuous batching of scene
// queries, one CUDA graph per batch.
//
// No reference counterpart: PoIntInt re-evaluates every object's form factors
// on every call (cpp/src/compute_intersection_volume_multi_object.cu:234-713,
// one kernel launch and k-grid upload per object).  Here:
//
//  * the library (elements + DoFs of every object a query may name) is
//    uploaded and prepared once, in each object's local frame;
//  * a pool of rows in HBM holds local-frame, direction-major, sqrt|w|-scaled
//    form factors: canonical rows (the object unrotated) stay resident under
//    an LRU policy within the HBM budget; a rotated object gets a row owned by
//    its batch (its form factors at R^T k);
//  * a translation never touches form factors: the contraction applies
//    e^{i k . c} with c = R o + t as it stages each row;
//  * a worker thread admits pending queries in arrival order into one of up
//    to four batch slots whenever a slot is free and the pool has room, so
//    queries that arrive while others run are admitted as slots and rows free
//    up, and batches on different slots overlap on the device;
//  * each batch is one graph launch on its slot's stream: descriptor upload,
//    form factors of the batch's new rows, the persistent tensor-core
//    contraction over every query of the batch, the split-K reduction, download
//    of results and row maxima.  Only the copy sizes, the form-factor grid and
//    whether that node runs change between launches of a slot's graph.
//
// A query's work items, k-chunk assignment and reduction order depend only on
// the query itself (its size and the autotuned items-per-SM of its size
// class), so its result is the same alone and in any mix.
#include <cuda.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>
#include "pi_internal.h"
#include "group.h"

using namespace pi;

namespace {

constexpr double INV_8PI3 = 1.0 / (8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846);
constexpr int MAX_SLOTS = 4;
constexpr int N_BUCKETS = 4;

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

int bucket_of(int n) { return n <= 16 ? 0 : n <= 128 ? 1 : n <= 512 ? 2 : 3; }

struct Ticket {
  uint64_t id = 0;
  int n = 0;
  std::vector<int32_t> obj;
  std::vector<double> rot;       // n x 9
  std::vector<uint8_t> rotated;  // per object
  std::vector<double> trans;     // n x 3
  double* V_out = nullptr;
  int state = PI_QUERY_PENDING;
  int status = PI_OK;
  std::string error;
  int64_t t_submit = 0, t_start = 0, t_done = 0;
  int64_t out_off = 0;           // doubles, within the slot's output region
};

// IO arena of a slot (device and pinned host mirror):
//   [header | queries | elem0 | evals | eval maxima | rows]  uploaded (prefix up to the used rows)
//   [error flag | outputs]                                    downloaded
// Each evaluation accumulates its row maximum into a zeroed slot of this
// arena; a commit kernel then copies it into the pool's persistent maxima,
// which every row descriptor points to.
struct Layout {
  size_t hdr, queries, elem0, evals, amax, rows, err, out, total;
};

struct Slot {
  int index = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  unsigned char* h_io = nullptr;
  unsigned char* d_io = nullptr;
  float* d_part = nullptr;
  int* d_err = nullptr;
  GroupDev g{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t n_h2d = nullptr, n_ff = nullptr, n_d2h_out = nullptr;
  bool ff_enabled = true;
  // current batch
  bool busy = false;
  uint64_t batch_id = 0;
  std::vector<uint64_t> tickets;
  std::vector<int> pins;         // pool rows pinned by this batch (one entry per pin)
  std::vector<int> temps;        // pool rows owned by this batch
  std::vector<int> produced;     // canonical rows evaluated by this batch
  int n_rows = 0, n_queries = 0, n_evals = 0;
  int64_t n_items = 0, n_out = 0;
};

struct Server {
  pi_kgrid_impl* kg = nullptr;
  int device = 0;
  pi_batch lib = nullptr;
  int n_lib = 0;
  std::vector<double> origin;    // 3 per library object
  pi_server_config cfg{};
  int op = GROUP_OP_F16;
  int sms = 148;
  int64_t Qpad = 0, nch = 0;
  int64_t max_items = 0, max_out = 0;
  Layout lay{};
  // pool
  float2* d_pool = nullptr;
  CUtensorMap pool_map;          // TMA view of the pool (tiles of consecutive rows load through it)
  float* d_pool_amax = nullptr;  // per pool row: max |Re|, |Im| (sets the FP16 operand scale)
  int64_t pool_rows = 0;
  std::vector<int> row_obj;      // canonical owner, or -1 (free) / -2 (batch-owned)
  std::vector<int> row_pin;
  std::vector<int> row_slot;     // slot whose batch evaluates the row, -1 when ready
  std::vector<uint64_t> row_batch;
  std::vector<int> free_rows;
  std::list<int> lru;            // resident canonical rows, least recently used first
  std::vector<std::list<int>::iterator> lru_pos;
  std::vector<uint8_t> in_lru;
  std::unordered_map<int, int> resident;  // library object -> pool row
  // slots
  Slot slots[MAX_SLOTS];
  int nslots = 2;
  uint64_t next_batch = 1;
  int tuned[N_BUCKETS] = {8, 8, 8, 8};  // work items per SM, in quarters
  // tickets
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> pending;
  std::unordered_map<uint64_t, std::unique_ptr<Ticket>> tickets;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::string fatal;             // set after a device failure: every later query fails with it
  std::thread worker;
  pi_server_stats st{};
};

// ---------------------------------------------------------------------------
// pool rows

void lru_touch(Server& S, int row) {
  if (S.in_lru[row]) S.lru.erase(S.lru_pos[row]);
  S.lru.push_back(row);
  S.lru_pos[row] = std::prev(S.lru.end());
  S.in_lru[row] = 1;
}

void lru_remove(Server& S, int row) {
  if (S.in_lru[row]) {
    S.lru.erase(S.lru_pos[row]);
    S.in_lru[row] = 0;
  }
}

// Whether `need` rows could be handed out now (free ones, then unpinned
// resident ones, least recently used first).
bool rows_available(const Server& S, int64_t need) {
  int64_t n = (int64_t)S.free_rows.size();
  if (n >= need) return true;
  for (int r : S.lru)
    if (S.row_pin[r] == 0 && S.row_slot[r] < 0 && ++n >= need) return true;
  return false;
}

int take_row(Server& S) {
  if (!S.free_rows.empty()) {
    const int r = S.free_rows.back();
    S.free_rows.pop_back();
    return r;
  }
  for (auto it = S.lru.begin(); it != S.lru.end(); ++it) {
    const int r = *it;
    if (S.row_pin[r] == 0 && S.row_slot[r] < 0) {
      S.lru.erase(it);
      S.in_lru[r] = 0;
      S.resident.erase(S.row_obj[r]);
      S.row_obj[r] = -1;
      ++S.st.evictions;
      return r;
    }
  }
  return -1;
}

// ---------------------------------------------------------------------------
// slot construction

Layout make_layout(const pi_server_config& c, int64_t max_out) {
  Layout L;
  L.hdr = 0;
  L.queries = 256;
  L.elem0 = al256(L.queries + (size_t)c.max_batch_queries * sizeof(GQuery));
  L.evals = al256(L.elem0 + (size_t)c.max_batch_queries * sizeof(int64_t));
  L.amax = al256(L.evals + (size_t)c.max_batch_evals * sizeof(EvalDev));
  L.rows = al256(L.amax + (size_t)c.max_batch_evals * sizeof(float));
  L.err = al256(L.rows + (size_t)c.max_batch_rows * sizeof(GRow));
  L.out = L.err + 256;
  L.total = al256(L.out + (size_t)max_out * sizeof(double));
  return L;
}

int build_graph(Server& S, Slot& sl) {
  PI_CUDA(cudaGraphCreate(&sl.graph, 0));
  // descriptor upload (size set per launch)
  cudaGraphNode_t n_err = nullptr, n_con = nullptr, n_red = nullptr;
  PI_CUDA(cudaGraphAddMemcpyNode1D(&sl.n_h2d, sl.graph, nullptr, 0, sl.d_io, sl.h_io, S.lay.rows,
                                   cudaMemcpyHostToDevice));
  cudaMemsetParams ms{};
  ms.dst = sl.d_err; ms.value = 0; ms.elementSize = 4; ms.width = 1; ms.height = 1; ms.pitch = 4;
  PI_CUDA(cudaGraphAddMemsetNode(&n_err, sl.graph, &sl.n_h2d, 1, &ms));
  // form factors of the batch's new rows (grid set per launch)
  KGridDev K = S.kg->dev;
  BatchDev B = S.lib->dev();
  float2* none = nullptr;
  int one = 1;
  EvalDev* evals = reinterpret_cast<EvalDev*>(sl.d_io + S.lay.evals);
  unsigned* no_amax = nullptr;  // serving rows keep their maxima through EvalDev::amax
  void* ff_args[6] = {&K, &B, &none, &one, &evals, &no_amax};
  cudaKernelNodeParams kp{};
  kp.func = const_cast<void*>(ff_serve_fn(S.kg));
  kp.gridDim = dim3((unsigned)ff_serve_grid_x(S.kg), 1);
  kp.blockDim = dim3((unsigned)ff_serve_threads());
  kp.sharedMemBytes = 0;
  kp.kernelParams = ff_args;
  PI_CUDA(cudaGraphAddKernelNode(&sl.n_ff, sl.graph, &n_err, 1, &kp));
  // row maxima of the new rows into the pool
  const int32_t* n_evals = &reinterpret_cast<const GHeader*>(sl.d_io + S.lay.hdr)->n_evals;
  void* cm_args[2] = {&evals, const_cast<int32_t**>(&n_evals)};
  cudaKernelNodeParams cmp{};
  cmp.func = const_cast<void*>(amax_commit_fn());
  cmp.gridDim = dim3(1);
  cmp.blockDim = dim3((unsigned)amax_commit_threads());
  cmp.kernelParams = cm_args;
  cudaGraphNode_t n_commit = nullptr;
  PI_CUDA(cudaGraphAddKernelNode(&n_commit, sl.graph, &sl.n_ff, 1, &cmp));
  // contraction
  void* con_args[2] = {&sl.g, &S.pool_map};
  cudaKernelNodeParams cpar{};
  cpar.func = const_cast<void*>(group_contract_fn(S.op, 1, 0));
  cpar.gridDim = dim3((unsigned)group_grid());
  cpar.blockDim = dim3((unsigned)group_threads());
  cpar.sharedMemBytes = (unsigned)group_smem_bytes();
  cpar.kernelParams = con_args;
  PI_CUDA(cudaGraphAddKernelNode(&n_con, sl.graph, &n_commit, 1, &cpar));
  // reduction
  void* red_args[1] = {&sl.g};
  cudaKernelNodeParams rp{};
  rp.func = const_cast<void*>(group_reduce_fn());
  rp.gridDim = dim3((unsigned)(4 * S.sms));
  rp.blockDim = dim3((unsigned)group_reduce_threads());
  rp.kernelParams = red_args;
  PI_CUDA(cudaGraphAddKernelNode(&n_red, sl.graph, &n_con, 1, &rp));
  // error flag + results download (size set per launch)
  PI_CUDA(cudaGraphAddMemcpyNode1D(&sl.n_d2h_out, sl.graph, &n_red, 1, sl.h_io + S.lay.err, sl.d_io + S.lay.err,
                                   256 + sizeof(double), cudaMemcpyDeviceToHost));
  PI_CUDA(cudaGraphInstantiate(&sl.exec, sl.graph, 0));
  return PI_OK;
}

int init_slot(Server& S, Slot& sl, int index) {
  sl.index = index;
  int lo = 0, hi = 0;
  PI_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  PI_CUDA(cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, hi));
  PI_CUDA(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
  PI_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&sl.h_io), S.lay.total, cudaHostAllocDefault));
  std::memset(sl.h_io, 0, S.lay.total);
  PI_CUDA(cudaMalloc(reinterpret_cast<void**>(&sl.d_io), S.lay.total));
  PI_CUDA(cudaMalloc(reinterpret_cast<void**>(&sl.d_part), (size_t)S.max_items * GROUP_TILE * GROUP_TILE * sizeof(float)));
  sl.d_err = reinterpret_cast<int*>(sl.d_io + S.lay.err);
  GroupDev& g = sl.g;
  g.hdr = reinterpret_cast<const GHeader*>(sl.d_io + S.lay.hdr);
  g.rows = reinterpret_cast<const GRow*>(sl.d_io + S.lay.rows);
  g.queries = reinterpret_cast<const GQuery*>(sl.d_io + S.lay.queries);
  g.elem0 = reinterpret_cast<const int64_t*>(sl.d_io + S.lay.elem0);
  g.ncols = S.Qpad;
  g.op = S.op;
  g.phase = 1;
  g.tile_tma = 1;
  g.L = S.kg->L;
  g.M = S.kg->M;
  g.dir_hi = S.kg->dev.dir_hi;
  g.dir_lo = S.kg->dev.dir_lo;
  g.kturn = S.kg->dev.kturn;
  g.partials = sl.d_part;
  g.max_items = S.max_items;
  g.err = sl.d_err;
  g.out = reinterpret_cast<double*>(sl.d_io + S.lay.out);
  g.scale = INV_8PI3;
  if (S.cfg.use_graphs) return build_graph(S, sl);
  return PI_OK;
}

// ---------------------------------------------------------------------------
// batch building (caller holds the lock)

// K splits of one query.  Rows are direction-major (L / 32 chunks per
// direction, one radial block each); the split stride is kept a multiple of
// L / 32 so that every work item stays inside one radial block.  Strides that
// mix radial blocks within an item raised the tensor-core contraction's error
// about five-fold on the 256-object scene (9e-5 against 2e-5, FP16 operands),
// for reasons this code does not rely on.
int nsplit_for(const Server& S, int n, int tuned_q4) {
  const int nt = (n + GROUP_TILE - 1) / GROUP_TILE;
  const int npairs = nt * (nt + 1) / 2;
  const int target = std::max(1, tuned_q4 * S.sms / 4);
  const int rb = std::max(1, S.kg->L / GROUP_CHUNK);
  // rounded down (to a multiple of rb, at least rb) so a query alone does not
  // leave a few CTAs with one item more than the rest
  int ns = std::max(1, target / npairs) / rb * rb;
  ns = std::max(ns, rb);
  return (int)std::min<int64_t>(ns, S.nch);
}

int nsplit_for(const Server& S, int n) { return nsplit_for(S, n, S.tuned[bucket_of(n)]); }

int64_t items_for(const Server& S, int n) {
  const int nt = (n + GROUP_TILE - 1) / GROUP_TILE;
  return (int64_t)nt * (nt + 1) / 2 * nsplit_for(S, n);
}

void split_df(double v, float* hi, float* lo) {
  *hi = (float)v;
  *lo = (float)(v - (double)*hi);
}

// Pool rows a query would take now: its rotated objects, plus its canonical
// objects that are neither resident nor already planned in this batch.
int64_t rows_needed(const Server& S, const Ticket& t, const std::unordered_map<int, int>& planned) {
  int64_t need = 0;
  std::vector<int> seen;
  for (int i = 0; i < t.n; ++i) {
    if (t.rotated[i]) { ++need; continue; }
    const int o = t.obj[i];
    if (S.resident.count(o) || planned.count(o)) continue;
    if (std::find(seen.begin(), seen.end(), o) != seen.end()) continue;
    seen.push_back(o);
    ++need;
  }
  return need;
}

void fail_ticket(Server& S, Ticket& t, int status, const std::string& msg) {
  t.state = PI_QUERY_FAILED;
  t.status = status;
  t.error = msg;
  t.t_done = now_ns();
  ++S.st.failed;
}

// Returns the number of queries admitted (0: nothing could be admitted now).
int build_batch(Server& S, Slot& sl, std::vector<cudaEvent_t>* waits) {
  const pi_server_config& c = S.cfg;
  GHeader* hdr = reinterpret_cast<GHeader*>(sl.h_io + S.lay.hdr);
  GQuery* qs = reinterpret_cast<GQuery*>(sl.h_io + S.lay.queries);
  int64_t* elem0 = reinterpret_cast<int64_t*>(sl.h_io + S.lay.elem0);
  EvalDev* evals = reinterpret_cast<EvalDev*>(sl.h_io + S.lay.evals);
  float* eval_amax = reinterpret_cast<float*>(sl.h_io + S.lay.amax);
  GRow* rows = reinterpret_cast<GRow*>(sl.h_io + S.lay.rows);
  float* d_eval_amax = reinterpret_cast<float*>(sl.d_io + S.lay.amax);
  sl.tickets.clear(); sl.pins.clear(); sl.temps.clear(); sl.produced.clear();
  sl.n_rows = sl.n_queries = sl.n_evals = 0;
  sl.n_items = sl.n_out = 0;
  int64_t n_elems = 0;
  std::unordered_map<int, int> planned;  // canonical object -> pool row evaluated by this batch
  std::vector<int> wait_slots;
  while (!S.pending.empty()) {
    Ticket& t = *S.tickets[S.pending.front()];
    if (t.state != PI_QUERY_PENDING) { S.pending.pop_front(); continue; }  // cancelled
    const int64_t need = rows_needed(S, t, planned);
    const int64_t new_evals = need;
    const int64_t items = items_for(S, t.n);
    const int64_t out = (int64_t)t.n * t.n;
    if (need > S.pool_rows || t.n > c.max_batch_rows || items > S.max_items || out > S.max_out ||
        new_evals > c.max_batch_evals) {
      fail_ticket(S, t, PI_ERR_WORKSPACE_TOO_SMALL, "query does not fit the server's pool or batch limits");
      S.pending.pop_front();
      continue;
    }
    if (sl.n_queries + 1 > c.max_batch_queries || sl.n_rows + t.n > c.max_batch_rows ||
        sl.n_evals + new_evals > c.max_batch_evals || sl.n_items + items > S.max_items || sl.n_out + out > S.max_out)
      break;  // admitted later, in arrival order
    // Pass 1: pin the resident rows the query reads (so that taking its new
    // rows cannot evict them), then check that the new rows can be had.
    std::vector<int> prow(t.n, -1);
    for (int i = 0; i < t.n; ++i) {
      if (t.rotated[i]) continue;
      auto it = S.resident.find(t.obj[i]);
      if (it != S.resident.end()) {
        prow[i] = it->second;
        S.row_pin[prow[i]]++;
      }
    }
    if (!rows_available(S, need)) {
      for (int i = 0; i < t.n; ++i)
        if (prow[i] >= 0) S.row_pin[prow[i]]--;
      break;  // rows free up as running batches retire
    }
    // Pass 2: admit.
    S.pending.pop_front();
    const int row0 = sl.n_rows;
    std::vector<int> qrow(t.n);
    for (int i = 0; i < t.n; ++i) {
      const int o = t.obj[i];
      int r = prow[i];
      auto add_eval = [&](int rot) {
        const int k = sl.n_evals++;
        EvalDev& e = evals[k];
        e.obj = o; e.rotate = rot;
        e.dst = S.d_pool + (int64_t)r * S.Qpad;
        eval_amax[k] = 0.f;
        e.amax = d_eval_amax + k;
        e.amax_keep = S.d_pool_amax + r;
        std::memcpy(e.R, &t.rot[9 * i], 9 * sizeof(double));
        ++S.st.evaluations;
      };
      if (t.rotated[i]) {
        r = take_row(S);
        S.row_obj[r] = -2;
        sl.temps.push_back(r);
        add_eval(1);
      } else if (r >= 0) {  // resident (pinned in pass 1)
        lru_touch(S, r);
        sl.pins.push_back(r);
        if (!planned.count(o)) {
          if (S.row_slot[r] >= 0) {  // evaluated by a batch still on the device
            const Slot& ps = S.slots[S.row_slot[r]];
            if (ps.busy && ps.batch_id == S.row_batch[r]) wait_slots.push_back(ps.index);
          }
          ++S.st.resident_hits;
        }
      } else {
        auto it = S.resident.find(o);  // an earlier object of this query may have made it resident
        if (it != S.resident.end()) {
          r = it->second;
        } else {
          r = take_row(S);
          S.row_obj[r] = o;
          S.resident[o] = r;
          S.row_slot[r] = sl.index;
          S.row_batch[r] = sl.batch_id;
          planned[o] = r;
          sl.produced.push_back(r);
          add_eval(0);
          ++S.st.resident_misses;
        }
        lru_touch(S, r);
        S.row_pin[r]++;
        sl.pins.push_back(r);
      }
      GRow& R = rows[sl.n_rows];
      R.J = S.d_pool + (int64_t)r * S.Qpad;
      R.amax = S.d_pool_amax + r;
      R.tma_row = -1;
      R.reserved_ = 0;
      qrow[i] = r;
      // centre c = R o + t
      const double* Rm = &t.rot[9 * i];
      const double* oo = &S.origin[3 * o];
      for (int a = 0; a < 3; ++a) {
        const double cv = Rm[3 * a] * oo[0] + Rm[3 * a + 1] * oo[1] + Rm[3 * a + 2] * oo[2] + t.trans[3 * i + a];
        split_df(cv, &R.c_hi[a], &R.c_lo[a]);
      }
      ++sl.n_rows;
    }
    // tiles whose rows are consecutive pool rows load by TMA
    for (int t0 = 0; t0 < t.n; t0 += GROUP_TILE) {
      const int na = std::min(GROUP_TILE, t.n - t0);
      bool run = true;
      for (int i = 1; i < na && run; ++i) run = qrow[t0 + i] == qrow[t0] + i;
      if (run) rows[row0 + t0].tma_row = qrow[t0];
    }
    GQuery& q = qs[sl.n_queries];
    q.row0 = row0;
    q.n = t.n;
    q.nt = (t.n + GROUP_TILE - 1) / GROUP_TILE;
    q.nsplit = nsplit_for(S, t.n);
    q.item0 = sl.n_items;
    q.out_off = sl.n_out;
    elem0[sl.n_queries] = n_elems;
    t.out_off = sl.n_out;
    t.state = PI_QUERY_RUNNING;
    t.t_start = now_ns();
    sl.tickets.push_back(t.id);
    ++sl.n_queries;
    sl.n_items += items;
    sl.n_out += out;
    n_elems += out;
  }
  if (sl.n_queries == 0) return 0;
  // Largest objects first: the evaluation grid's CTAs start in this order, so
  // a large object's CTAs do not start last and leave the SMs idle at the end
  // (each evaluation carries its own destination row and row-maximum slots).
  std::stable_sort(evals, evals + sl.n_evals, [&](const EvalDev& x, const EvalDev& y) {
    return S.lib->info[x.obj].n_elems > S.lib->info[y.obj].n_elems;
  });
  hdr->n_items = (int32_t)sl.n_items;
  hdr->n_queries = sl.n_queries;
  hdr->n_elems = n_elems;
  hdr->n_evals = sl.n_evals;
  hdr->reserved_ = 0;
  std::sort(wait_slots.begin(), wait_slots.end());
  wait_slots.erase(std::unique(wait_slots.begin(), wait_slots.end()), wait_slots.end());
  for (int w : wait_slots) waits->push_back(S.slots[w].done);
  return sl.n_queries;
}

int launch_batch(Server& S, Slot& sl, const std::vector<cudaEvent_t>& waits) {
  for (cudaEvent_t e : waits) PI_CUDA(cudaStreamWaitEvent(sl.stream, e, 0));
  const size_t h2d = S.lay.rows + (size_t)sl.n_rows * sizeof(GRow);
  const size_t out_bytes = 256 + (size_t)std::max<int64_t>(1, sl.n_out) * sizeof(double);  // flag + results
  if (S.cfg.use_graphs) {
    PI_CUDA(cudaGraphExecMemcpyNodeSetParams1D(sl.exec, sl.n_h2d, sl.d_io, sl.h_io, h2d, cudaMemcpyHostToDevice));
    const bool ff = sl.n_evals > 0;
    if (ff) {
      KGridDev K = S.kg->dev;
      BatchDev B = S.lib->dev();
      float2* none = nullptr;
      int one = 1;
      EvalDev* evals = reinterpret_cast<EvalDev*>(sl.d_io + S.lay.evals);
      unsigned* no_amax = nullptr;
      void* ff_args[6] = {&K, &B, &none, &one, &evals, &no_amax};
      cudaKernelNodeParams kp{};
      kp.func = const_cast<void*>(ff_serve_fn(S.kg));
      kp.gridDim = dim3((unsigned)ff_serve_grid_x(S.kg), (unsigned)sl.n_evals);
      kp.blockDim = dim3((unsigned)ff_serve_threads());
      kp.kernelParams = ff_args;
      PI_CUDA(cudaGraphExecKernelNodeSetParams(sl.exec, sl.n_ff, &kp));
    }
    if (ff != sl.ff_enabled) {
      PI_CUDA(cudaGraphNodeSetEnabled(sl.exec, sl.n_ff, ff ? 1u : 0u));
      sl.ff_enabled = ff;
    }
    PI_CUDA(cudaGraphExecMemcpyNodeSetParams1D(sl.exec, sl.n_d2h_out, sl.h_io + S.lay.err, sl.d_io + S.lay.err,
                                               out_bytes, cudaMemcpyDeviceToHost));
    PI_CUDA(cudaGraphLaunch(sl.exec, sl.stream));
    ++S.st.graph_launches;
  } else {
    PI_CUDA(cudaMemcpyAsync(sl.d_io, sl.h_io, h2d, cudaMemcpyHostToDevice, sl.stream));
    PI_CUDA(cudaMemsetAsync(sl.d_err, 0, sizeof(int), sl.stream));
    int rc = launch_form_factors_serve(S.kg, S.lib, reinterpret_cast<EvalDev*>(sl.d_io + S.lay.evals), sl.n_evals,
                                       sl.stream);
    if (rc) return rc;
    rc = launch_amax_commit(reinterpret_cast<EvalDev*>(sl.d_io + S.lay.evals),
                            &reinterpret_cast<const GHeader*>(sl.d_io + S.lay.hdr)->n_evals, sl.stream);
    if (rc) return rc;
    rc = launch_group_contract(sl.g, &S.pool_map, false, group_grid(), sl.stream);
    if (rc) return rc;
    rc = launch_group_reduce(sl.g, 4 * S.sms, sl.stream);
    if (rc) return rc;
    PI_CUDA(cudaMemcpyAsync(sl.h_io + S.lay.err, sl.d_io + S.lay.err, out_bytes, cudaMemcpyDeviceToHost, sl.stream));
  }
  PI_CUDA(cudaEventRecord(sl.done, sl.stream));
  ++S.st.batches;
  return PI_OK;
}

void release_batch_rows(Server& S, Slot& sl) {
  for (int r : sl.pins) S.row_pin[r]--;
  for (int r : sl.temps) {
    S.row_obj[r] = -1;
    S.free_rows.push_back(r);
  }
  for (int r : sl.produced)
    if (S.row_slot[r] == sl.index && S.row_batch[r] == sl.batch_id) S.row_slot[r] = -1;
}

// A batch's queries fail and the rows it was evaluating are dropped.
void abort_batch(Server& S, Slot& sl, int status, const std::string& msg) {
  for (int r : sl.produced) {
    if (S.row_obj[r] >= 0) S.resident.erase(S.row_obj[r]);
    lru_remove(S, r);
    S.row_obj[r] = -2;  // returned to the free list below, with the temps
    sl.temps.push_back(r);
  }
  release_batch_rows(S, sl);
  for (uint64_t id : sl.tickets) {
    auto it = S.tickets.find(id);
    if (it != S.tickets.end()) fail_ticket(S, *it->second, status, msg);
  }
  sl.busy = false;
  S.cv_done.notify_all();
}

void retire_batch(Server& S, Slot& sl) {
  const double* out = reinterpret_cast<const double*>(sl.h_io + S.lay.out);
  const int err = *reinterpret_cast<const int*>(sl.h_io + S.lay.err);
  release_batch_rows(S, sl);
  const int64_t t = now_ns();
  for (uint64_t id : sl.tickets) {
    auto it = S.tickets.find(id);
    if (it == S.tickets.end()) continue;
    Ticket& tk = *it->second;
    const int64_t nn = (int64_t)tk.n * tk.n;
    if (err != 0) {
      fail_ticket(S, tk, PI_ERR_CUDA, "the contraction reported an error (bounded wait expired)");
      continue;
    }
    if (tk.V_out) std::memcpy(tk.V_out, out + tk.out_off, (size_t)nn * sizeof(double));
    tk.state = PI_QUERY_DONE;
    tk.t_done = t;
    ++S.st.completed;
  }
  sl.busy = false;
  S.cv_done.notify_all();
}

void worker_loop(Server* Sp) {
  Server& S = *Sp;
  cudaSetDevice(S.device);
  std::unique_lock<std::mutex> lk(S.mu);
  while (true) {
    // retire finished batches
    bool any_busy = false;
    for (int i = 0; i < S.nslots; ++i) {
      Slot& sl = S.slots[i];
      if (!sl.busy) continue;
      const cudaError_t e = cudaEventQuery(sl.done);
      if (e == cudaSuccess) retire_batch(S, sl);
      else if (e != cudaErrorNotReady) {
        S.fatal = std::string("device failure: ") + cudaGetErrorString(e);
        abort_batch(S, sl, PI_ERR_CUDA, S.fatal);
      } else any_busy = true;
    }
    if (!S.fatal.empty()) {
      while (!S.pending.empty()) {
        auto it = S.tickets.find(S.pending.front());
        if (it != S.tickets.end() && it->second->state == PI_QUERY_PENDING) fail_ticket(S, *it->second, PI_ERR_CUDA, S.fatal);
        S.pending.pop_front();
      }
      S.cv_done.notify_all();
    }
    if (S.stop && S.pending.empty() && !any_busy) break;
    // admit into a free slot
    bool launched = false;
    if (!S.pending.empty() && S.fatal.empty()) {
      for (int i = 0; i < S.nslots && !launched; ++i) {
        Slot& sl = S.slots[i];
        if (sl.busy) continue;
        sl.batch_id = S.next_batch++;
        std::vector<cudaEvent_t> waits;
        if (build_batch(S, sl, &waits) == 0) { S.cv_done.notify_all(); break; }
        sl.busy = true;
        const int rc = launch_batch(S, sl, waits);
        if (rc != PI_OK) {
          S.fatal = std::string("batch launch failed: ") + pi_last_error();
          abort_batch(S, sl, rc, S.fatal);
        }
        launched = true;
      }
    }
    if (launched) continue;
    bool busy_now = false;
    for (int i = 0; i < S.nslots; ++i) busy_now |= S.slots[i].busy;
    if (busy_now) S.cv_work.wait_for(lk, std::chrono::microseconds(20));
    else if (S.pending.empty() && !S.stop) S.cv_work.wait_for(lk, std::chrono::milliseconds(50));
    else if (!S.pending.empty()) S.cv_work.wait_for(lk, std::chrono::microseconds(200));  // head does not fit yet
  }
}

// ---------------------------------------------------------------------------
// autotuning of work items per SM (one query alone, direct launches)

__attribute__((unused)) void fill_rows_host(std::vector<float2>& h, int64_t n, uint64_t seed) {
  uint64_t x = seed;
  for (int64_t i = 0; i < n; ++i) {
    x = x * 6364136223846793005ULL + 1442695040888963407ULL;
    const float a = (float)((x >> 40) & 0xffff) / 65536.f - 0.5f;
    const float b = (float)((x >> 20) & 0xffff) / 65536.f - 0.5f;
    h[i] = make_float2(a, b);
  }
}

int autotune(Server& S) {
  const int sizes[3] = {16, 128, 512};
  const int cand[4] = {2, 4, 8, 16};  // items per SM, quarters: 0.5x .. 4x
  const int64_t rows = std::min<int64_t>(512, S.pool_rows);
  if (rows < 16) return PI_OK;
  // synthetic rows (the pool is zeroed again afterwards)
  std::vector<float2> h((size_t)(S.Qpad));
  for (int64_t r = 0; r < rows; ++r) {
    fill_rows_host(h, S.kg->Q, 1234567 + r);  // padding columns stay zero
    PI_CUDA(cudaMemcpy(S.d_pool + r * S.Qpad, h.data(), (size_t)S.Qpad * sizeof(float2), cudaMemcpyHostToDevice));
  }
  Slot& sl = S.slots[0];
  GHeader* hdr = reinterpret_cast<GHeader*>(sl.h_io + S.lay.hdr);
  GQuery* qs = reinterpret_cast<GQuery*>(sl.h_io + S.lay.queries);
  int64_t* elem0 = reinterpret_cast<int64_t*>(sl.h_io + S.lay.elem0);
  GRow* rw = reinterpret_cast<GRow*>(sl.h_io + S.lay.rows);
  cudaEvent_t a, b;
  PI_CUDA(cudaEventCreate(&a));
  PI_CUDA(cudaEventCreate(&b));
  for (int si = 0; si < 3; ++si) {
    const int n = (int)std::min<int64_t>(sizes[si], rows);
    // a batch of nq copies of the scene: the setting has to serve loaded batches, not one query alone
    const int nq = std::max(1, std::min({4, S.cfg.max_batch_queries, S.cfg.max_batch_rows / std::max(1, n)}));
    if (n * nq > S.cfg.max_batch_rows || (int64_t)n * n * nq > S.max_out) continue;
    float best = 1e30f;
    int best_c = S.tuned[si];
    for (int c : cand) {
      const int nt = (n + GROUP_TILE - 1) / GROUP_TILE, npairs = nt * (nt + 1) / 2;
      const int ns = nsplit_for(S, n, c);
      if ((int64_t)npairs * ns * nq > S.max_items) continue;
      for (int i = 0; i < n * nq; ++i) {
        rw[i].J = S.d_pool + (int64_t)(i % n) * S.Qpad;
        rw[i].amax = S.d_pool_amax + (i % n);
        rw[i].tma_row = -1;
        rw[i].reserved_ = 0;
        for (int k = 0; k < 3; ++k) split_df(0.37 * (i % 7) - 0.9 * k, &rw[i].c_hi[k], &rw[i].c_lo[k]);
      }
      for (int j = 0; j < nq; ++j) {
        qs[j].row0 = j * n; qs[j].n = n; qs[j].nt = nt; qs[j].nsplit = ns;
        qs[j].item0 = (int64_t)j * npairs * ns; qs[j].out_off = (int64_t)j * n * n;
        elem0[j] = (int64_t)j * n * n;
      }
      hdr->n_items = npairs * ns * nq; hdr->n_queries = nq; hdr->n_elems = (int64_t)n * n * nq; hdr->n_evals = 0;
      PI_CUDA(cudaMemcpyAsync(sl.d_io, sl.h_io, S.lay.rows + (size_t)n * nq * sizeof(GRow), cudaMemcpyHostToDevice,
                              sl.stream));
      float t_min = 1e30f;
      for (int rep = 0; rep < 4; ++rep) {
        PI_CUDA(cudaMemsetAsync(sl.d_err, 0, sizeof(int), sl.stream));
        PI_CUDA(cudaEventRecord(a, sl.stream));
        int rc = launch_group_contract(sl.g, &S.pool_map, false, group_grid(), sl.stream);
        if (rc) return rc;
        rc = launch_group_reduce(sl.g, 4 * S.sms, sl.stream);
        if (rc) return rc;
        PI_CUDA(cudaEventRecord(b, sl.stream));
        PI_CUDA(cudaEventSynchronize(b));
        float ms = 0.f;
        PI_CUDA(cudaEventElapsedTime(&ms, a, b));
        if (rep > 0) t_min = std::min(t_min, ms);
      }
      int herr = 0;
      PI_CUDA(cudaMemcpy(&herr, sl.d_err, sizeof(int), cudaMemcpyDeviceToHost));
      if (herr) return fail(PI_ERR_CUDA, "autotuning run reported a device error");
      if (t_min < best) { best = t_min; best_c = c; }
    }
    S.tuned[si] = best_c;
    if (si == 2) S.tuned[3] = best_c;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  PI_CUDA(cudaMemset(S.d_pool, 0, (size_t)rows * S.Qpad * sizeof(float2)));
  PI_CUDA(cudaMemset(S.d_pool_amax, 0, (size_t)rows * sizeof(float)));
  return PI_OK;
}

void destroy_server(Server* S) {
  if (!S) return;
  for (int i = 0; i < MAX_SLOTS; ++i) {
    Slot& sl = S->slots[i];
    if (sl.exec) cudaGraphExecDestroy(sl.exec);
    if (sl.graph) cudaGraphDestroy(sl.graph);
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.h_io) cudaFreeHost(sl.h_io);
    if (sl.d_io) cudaFree(sl.d_io);
    if (sl.d_part) cudaFree(sl.d_part);
  }
  if (S->d_pool) cudaFree(S->d_pool);
  if (S->d_pool_amax) cudaFree(S->d_pool_amax);
  if (S->lib) pi_batch_destroy(S->lib);
  delete S;
}

}  // namespace

struct pi_server_s : Server {};

extern "C" {

int pi_server_create(pi_kgrid kg, const pi_object* library, int n_library, const pi_server_config* cfg_in,
                     pi_server* out) {
  if (!out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_create: null output");
  *out = nullptr;
  if (!kg || n_library <= 0 || !library) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_create: empty library");
  if (!kg->tensor || kg->L % 16 != 0 || kg->L > GROUP_MAX_L)
    return fail(PI_ERR_UNSUPPORTED,
                "the serving path needs a Gauss-Legendre x Lebedev k-grid with a multiple of 16 radial nodes (<= 512)");
  if (!kg->all_positive) return fail(PI_ERR_UNSUPPORTED, "the serving path needs non-negative quadrature weights");
  if (kg->Q >= (int64_t(1) << 31) - 64) return fail(PI_ERR_UNSUPPORTED, "the serving path supports fewer than 2^31 k-nodes");
  pi_server_config c{};
  if (cfg_in) c = *cfg_in;
  if (c.max_batch_queries <= 0) c.max_batch_queries = 64;
  if (c.max_batch_rows <= 0) c.max_batch_rows = 4096;
  if (c.max_batch_evals <= 0) c.max_batch_evals = 256;
  // four batches in flight: with two, the worker's retire-and-build between
  // batches left the device idle (256-object scenes: 7.2k vs 10.3k matrices/s)
  if (c.inflight_batches <= 0) c.inflight_batches = MAX_SLOTS;
  if (c.inflight_batches > MAX_SLOTS) c.inflight_batches = MAX_SLOTS;
  if (c.precision == 0) c.precision = PI_CONTRACT_FP16X3;
  if (c.precision != PI_CONTRACT_FP16X3 && c.precision != PI_CONTRACT_BF16X3)
    return fail(PI_ERR_UNSUPPORTED, "the serving path computes in FP16X3 or BF16X3");
  if (c.use_graphs < 0) c.use_graphs = 1;
  if (c.autotune < 0) c.autotune = 1;
  if (c.max_batch_evals > 65535) c.max_batch_evals = 65535;
  std::unique_ptr<pi_server_s> S(new pi_server_s());
  S->kg = kg;
  S->cfg = c;
  S->op = c.precision == PI_CONTRACT_BF16X3 ? GROUP_OP_BF16 : GROUP_OP_F16;
  S->nslots = c.inflight_batches;
  S->n_lib = n_library;
  PI_CUDA(cudaGetDevice(&S->device));
  PI_CUDA(cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, S->device));
  S->Qpad = (kg->Q + GROUP_CHUNK - 1) / GROUP_CHUNK * GROUP_CHUNK;
  S->nch = S->Qpad / GROUP_CHUNK;
  // library: uploaded and prepared once
  int rc = pi_batch_create(library, n_library, 0, nullptr, &S->lib);
  if (rc) return rc;
  rc = pi_batch_prepare(S->lib, nullptr);
  if (rc) return rc;
  std::vector<ObjDev> od(n_library);
  PI_CUDA(cudaMemcpy(od.data(), S->lib->d_objs, sizeof(ObjDev) * n_library, cudaMemcpyDeviceToHost));
  S->origin.resize(3 * (size_t)n_library);
  for (int i = 0; i < n_library; ++i)
    for (int a = 0; a < 3; ++a) S->origin[3 * i + a] = od[i].origin[a];
  // arenas: items for the largest admissible batch (every row in 1-object
  // queries is the worst case for items per row)
  S->max_out = std::max<int64_t>((int64_t)c.max_batch_rows * 128, 512 * 512);
  int64_t per_query_max = 0;
  for (int n : {1, 16, 128, 256, 512, 1024, c.max_batch_rows}) {
    if (n > c.max_batch_rows) continue;
    const int nt = (n + GROUP_TILE - 1) / GROUP_TILE;
    const int q4 = std::max(16, std::min(c.items_per_sm_x4, 64));
    const int rb = std::max(1, kg->L / GROUP_CHUNK);
    const int64_t ns = std::min<int64_t>(S->nch, ((std::max(1, (q4 * S->sms / 4 + nt * (nt + 1) / 2 - 1) / (nt * (nt + 1) / 2)) + rb - 1) / rb) * rb);
    const int64_t items = (int64_t)nt * (nt + 1) / 2 * ns;
    per_query_max = std::max(per_query_max, items);
  }
  S->max_items = std::min<int64_t>((int64_t)c.max_batch_queries * std::max(16, std::min(c.items_per_sm_x4, 64)) / 4 * S->sms,
                                  8 * per_query_max);
  S->max_items = std::max(S->max_items, per_query_max);
  S->lay = make_layout(c, S->max_out);
  const size_t slot_bytes = S->lay.total + (size_t)S->max_items * GROUP_TILE * GROUP_TILE * sizeof(float) + 256;
  size_t free_b = 0, total_b = 0;
  PI_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const int64_t budget = c.hbm_budget_bytes > 0 ? c.hbm_budget_bytes : (int64_t)(free_b / 4);
  const int64_t row_bytes = S->Qpad * (int64_t)sizeof(float2);
  const int64_t pool_bytes = budget - (int64_t)slot_bytes * S->nslots;
  if (pool_bytes < row_bytes * 2)
    return fail(PI_ERR_OUT_OF_MEMORY, "pi_server_create: HBM budget leaves no room for resident rows");
  S->pool_rows = std::min<int64_t>(pool_bytes / row_bytes, 0x7fffffff);
  PI_CUDA(cudaMalloc(reinterpret_cast<void**>(&S->d_pool), (size_t)(S->pool_rows * row_bytes)));
  PI_CUDA(cudaMemset(S->d_pool, 0, (size_t)(S->pool_rows * row_bytes)));
  S->row_obj.assign(S->pool_rows, -1);
  S->row_pin.assign(S->pool_rows, 0);
  rc = encode_row_map(&S->pool_map, S->d_pool, 2 * S->Qpad, S->pool_rows);
  if (rc) return rc;
  PI_CUDA(cudaMalloc(reinterpret_cast<void**>(&S->d_pool_amax), (size_t)S->pool_rows * sizeof(float)));
  PI_CUDA(cudaMemset(S->d_pool_amax, 0, (size_t)S->pool_rows * sizeof(float)));
  S->row_slot.assign(S->pool_rows, -1);
  S->row_batch.assign(S->pool_rows, 0);
  S->lru_pos.resize(S->pool_rows);
  S->in_lru.assign(S->pool_rows, 0);
  S->free_rows.reserve(S->pool_rows);
  for (int64_t r = S->pool_rows - 1; r >= 0; --r) S->free_rows.push_back((int)r);
  rc = group_prepare_attributes();
  if (rc) return rc;
  for (int i = 0; i < S->nslots; ++i) {
    rc = init_slot(*S, S->slots[i], i);
    if (rc) { destroy_server(S.release()); return rc; }
  }
  if (c.items_per_sm_x4 > 0) {
    for (int i = 0; i < N_BUCKETS; ++i) S->tuned[i] = std::min(c.items_per_sm_x4, 64);
  } else if (c.autotune) {
    rc = autotune(*S);
    if (rc) { destroy_server(S.release()); return rc; }
  }
  S->st.pool_rows = S->pool_rows;
  S->worker = std::thread(worker_loop, static_cast<Server*>(S.get()));
  *out = S.release();
  return PI_OK;
}

int pi_server_submit(pi_server s, const pi_query* q, double* V_out, uint64_t* ticket) {
  if (!s || !q || !ticket || q->n_objects <= 0 || !q->objects)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_submit: bad arguments");
  const int n = q->n_objects;
  std::unique_ptr<Ticket> t(new Ticket());
  t->n = n;
  t->obj.assign(q->objects, q->objects + n);
  t->rot.assign(9 * (size_t)n, 0.0);
  t->rotated.assign(n, 0);
  t->trans.assign(3 * (size_t)n, 0.0);
  for (int i = 0; i < n; ++i) {
    if (t->obj[i] < 0 || t->obj[i] >= s->n_lib) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_submit: object index out of range");
    double* R = &t->rot[9 * i];
    R[0] = R[4] = R[8] = 1.0;
    if (q->rotations) {
      const double* Rq = q->rotations + 9 * (size_t)i;
      // proper rotation: R R^T = I and det R = 1, to 1e-9
      double err = 0.0;
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          double d = 0.0;
          for (int k = 0; k < 3; ++k) d += Rq[3 * a + k] * Rq[3 * b + k];
          err = std::max(err, std::fabs(d - (a == b ? 1.0 : 0.0)));
        }
      const double det = Rq[0] * (Rq[4] * Rq[8] - Rq[5] * Rq[7]) - Rq[1] * (Rq[3] * Rq[8] - Rq[5] * Rq[6]) +
                         Rq[2] * (Rq[3] * Rq[7] - Rq[4] * Rq[6]);
      if (!(err <= 1e-9) || !(std::fabs(det - 1.0) <= 1e-9))
        return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_submit: rotations must be proper orthogonal matrices");
      bool identity = true;
      for (int k = 0; k < 9; ++k) identity &= Rq[k] == ((k % 4 == 0) ? 1.0 : 0.0);
      if (!identity) {
        std::memcpy(R, Rq, 9 * sizeof(double));
        t->rotated[i] = 1;
      }
    }
    if (q->translations)
      for (int a = 0; a < 3; ++a) {
        t->trans[3 * i + a] = q->translations[3 * (size_t)i + a];
        if (!std::isfinite(t->trans[3 * i + a])) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_submit: non-finite translation");
      }
  }
  t->V_out = V_out;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return fail(PI_ERR_UNSUPPORTED, "pi_server_submit: the server is shutting down");
  t->id = s->next_ticket++;
  t->t_submit = now_ns();
  *ticket = t->id;
  ++s->st.submitted;
  if (!s->fatal.empty()) {
    fail_ticket(*s, *t, PI_ERR_CUDA, s->fatal);
  } else {
    s->pending.push_back(t->id);
  }
  s->tickets[t->id] = std::move(t);
  s->cv_work.notify_one();
  return PI_OK;
}

int pi_server_poll(pi_server s, uint64_t ticket, int32_t* state) {
  if (!s || !state) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_poll: bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return fail(PI_ERR_NOT_FOUND, "pi_server_poll: unknown ticket");
  *state = it->second->state;
  return PI_OK;
}

int pi_server_wait(pi_server s, uint64_t ticket, double timeout_s) {
  if (!s) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_wait: null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto done = [&] {
    auto it = s->tickets.find(ticket);
    return it == s->tickets.end() || it->second->state >= PI_QUERY_DONE;
  };
  if (timeout_s < 0) s->cv_done.wait(lk, done);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
    return fail(PI_ERR_TIMEOUT, "pi_server_wait: timed out");
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return fail(PI_ERR_NOT_FOUND, "pi_server_wait: unknown ticket");
  const Ticket& t = *it->second;
  if (t.state == PI_QUERY_DONE) return PI_OK;
  if (t.state == PI_QUERY_CANCELLED) return fail(PI_ERR_NOT_FOUND, "pi_server_wait: the query was cancelled");
  return fail(t.status ? t.status : PI_ERR_CUDA, t.error);
}

int pi_server_cancel(pi_server s, uint64_t ticket) {
  if (!s) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_cancel: null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return fail(PI_ERR_NOT_FOUND, "pi_server_cancel: unknown ticket");
  Ticket& t = *it->second;
  if (t.state != PI_QUERY_PENDING) return fail(PI_ERR_UNSUPPORTED, "pi_server_cancel: the query is already running or finished");
  t.state = PI_QUERY_CANCELLED;
  t.t_done = now_ns();
  ++s->st.cancelled;
  s->cv_done.notify_all();
  return PI_OK;
}

int pi_server_times(pi_server s, uint64_t ticket, int64_t* submit_ns, int64_t* start_ns, int64_t* done_ns) {
  if (!s) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_times: null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return fail(PI_ERR_NOT_FOUND, "pi_server_times: unknown ticket");
  if (submit_ns) *submit_ns = it->second->t_submit;
  if (start_ns) *start_ns = it->second->t_start;
  if (done_ns) *done_ns = it->second->t_done;
  return PI_OK;
}

int pi_server_release(pi_server s, uint64_t ticket) {
  if (!s) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_release: null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return fail(PI_ERR_NOT_FOUND, "pi_server_release: unknown ticket");
  if (it->second->state < PI_QUERY_DONE) return fail(PI_ERR_UNSUPPORTED, "pi_server_release: the query has not finished");
  s->tickets.erase(it);
  return PI_OK;
}

int pi_server_stats_get(pi_server s, pi_server_stats* out) {
  if (!s || !out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_server_stats_get: bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  pi_server_stats st = s->st;
  st.pool_rows = s->pool_rows;
  st.resident_rows = (int64_t)s->resident.size();
  for (int i = 0; i < 4; ++i) st.tuned_items_per_sm[i] = s->tuned[i];
  const int rep_n[4] = {16, 128, 512, 1024};
  for (int i = 0; i < 4; ++i) st.tuned_k_splits[i] = nsplit_for(*s, rep_n[i]);
  *out = st;
  return PI_OK;
}

int pi_server_destroy(pi_server s) {
  if (!s) return PI_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (uint64_t id : s->pending) {
      auto it = s->tickets.find(id);
      if (it != s->tickets.end() && it->second->state == PI_QUERY_PENDING)
        fail_ticket(*s, *it->second, PI_ERR_UNSUPPORTED, "the server was destroyed");
    }
    s->pending.clear();
    s->cv_done.notify_all();
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  destroy_server(s);
  return PI_OK;
}

}  // extern "C"
