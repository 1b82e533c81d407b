// serve_host.cu — K9 host engine: the pricing server.
//
// One host thread per server drives the device in ticks.  Each tick it
//   1. admits queued requests into free slots while the memory budget allows
//      (a request reserves its slot record and the chunk partials of its
//      largest slice in every tick buffer);
//   2. plans the tick: every scheduled slot contributes one slice of its
//      current phase (min(slice, remaining) paths; the slice size is a
//      function of the request alone), in FIFO or shortest-remaining order up
//      to the tick's work cap; entries are grouped by kernel class;
//   3. enqueues: one copy of the plan and of the staged slot records, the
//      install kernel, the class kernels (spread over side streams), the
//      per-slot reduction and one copy of the finished-phase records back;
//   4. while that tick runs, waits for the previous one and handles its
//      finished phases: a pilot sizes the main run (find_num_trials,
//      sde_mc/mc.py:418-427) and fits the control-variate coefficients; a
//      main run becomes a result.
// kTickBufs tick buffers rotate, each with its own stream and side streams,
// so up to kTickBufs ticks are in flight: the next ticks are queued before the
// running one ends and their class kernels start while the running tick's
// last kernels drain: a class kernel reads only
// its entries and the slots' descriptors and coefficients (no running tick
// writes those), and the one ordering across ticks — each slot's FP64 sums are
// folded tick after tick — is kept by making each tick's reduction wait for
// the previous tick's.  The device busy time is the union of the ticks'
// intervals on one device timeline.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "serve_kernels.cuh"

namespace sdemc {

namespace {

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

constexpr int kNumClassKeys = kNumKinds * 3 * 2 * SDEMC_MAX_DIM;
constexpr int64_t kMaxSlicePaths = 1 << 18;
constexpr int64_t kMinSlicePaths = 1 << 10;
constexpr double kZ95 = 1.96;
constexpr int kTickBufs = 4;  // ticks in flight at most

bool lcv_supported(const sdemc_inst& I) {
  return I.noise == SDEMC_NOISE_DIAG && !(I.flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP);
}

int loop_mode_of(const sdemc_inst& I) {
  return (I.flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP) ? kModeNominal : 0;
}

int class_key(int kind, const sdemc_inst& I) {
  return ((kind * 3 + I.noise) * 2 + (loop_mode_of(I) == kModeNominal ? 1 : 0)) * SDEMC_MAX_DIM + (I.dim - 1);
}

// Expected work of one path in path-step x dim units (executed steps of the
// jump-adapted grid: nominal steps plus the expected number of jumps).
double path_cost(const sdemc_inst& I) {
  double steps = (double)I.num_steps;
  if (I.grid == SDEMC_GRID_ADAPTED) steps += (double)I.rate * (double)I.T;
  return steps * (double)I.dim;
}

// Solve C beta = c for a symmetric positive semi-definite C (d <= 16) by
// Cholesky with a small diagonal jitter; returns false if C is degenerate.
// A regressor that is identically zero gets a zero coefficient.
bool solve_spd(int d, const double* C, const double* c, double* beta) {
  double L[kServeMaxR][kServeMaxR] = {};
  double tr = 0.0;
  for (int i = 0; i < d; ++i) tr += C[i * d + i];
  if (!(tr > 0.0) || !std::isfinite(tr)) return false;
  const double jitter = 1e-12 * tr / d;
  for (int i = 0; i < d; ++i) {
    for (int j = 0; j <= i; ++j) {
      double s = C[i * d + j] + (i == j ? jitter : 0.0);
      for (int k = 0; k < j; ++k) s -= L[i][k] * L[j][k];
      if (i == j) {
        if (!(s > 0.0)) return false;
        L[i][i] = std::sqrt(s);
      } else {
        L[i][j] = s / L[j][j];
      }
    }
  }
  double z[kServeMaxR];
  for (int i = 0; i < d; ++i) {
    double s = c[i];
    for (int k = 0; k < i; ++k) s -= L[i][k] * z[k];
    z[i] = s / L[i][i];
  }
  for (int i = d - 1; i >= 0; --i) {
    double s = z[i];
    for (int k = i + 1; k < d; ++k) s -= L[k][i] * beta[k];
    beta[i] = s / L[i][i];
  }
  for (int i = 0; i < d; ++i)
    if (!std::isfinite(beta[i])) return false;
  return true;
}

struct Pending {
  sdemc_request req;
  int64_t t_arrive;
};

struct HostSlot {
  bool used = false;
  bool awaiting = false;  // a phase ends in a tick that has not been read back
  sdemc_request req;
  int64_t t_arrive = 0, t_admit = 0;
  uint64_t seq = 0;
  int phase = 0, kind = 0, width = 3, est = SDEMC_EST_PLAIN;
  int64_t cursor = 0, phase_end = 0, slice = 0, reserve = 0, pilot_paths = 0;
  double cost = 0.0, pilot_mean = 0.0, pilot_se = 0.0, vrf = 1.0;
  float beta[kServeMaxR] = {};
  CvWeights cw{};
};

struct TickBuf {
  cudaStream_t stream = nullptr;          // the tick's own stream
  std::vector<cudaStream_t> side;         // class kernels spread over these
  cudaEvent_t fork = nullptr, red_done = nullptr;
  std::vector<cudaEvent_t> join;
  int64_t seq = -1;                       // tick number (index into the end-stamp ring)
  ServeEntry* entries_h = nullptr;
  ServeInstall* installs_h = nullptr;
  ServeDone* done_h = nullptr;
  ServeEntry* entries_d = nullptr;
  ServeInstall* installs_d = nullptr;
  ServeDone* done_d = nullptr;
  unsigned long long* counters_d = nullptr;
  double* part_d = nullptr;
  cudaEvent_t t0 = nullptr;  // tick start (the end is its stamp in the ring)
  int n_entries = 0, n_installs = 0, n_done = 0, launches = 0;
  double path_steps = 0.0;
};

}  // namespace

// The control variate's integrand weight for a descriptor (see CvWeights):
// a Black-Scholes call (or put) delta of the payoff's underlying with the
// lognormal volatility of that underlying, jumps included.  Any choice keeps
// the estimator unbiased; a good one makes the variance reduction large.
CvWeights serve_cv_weights(const sdemc_inst& I) {
  CvWeights cw{};
  const int d = I.dim;
  double jump_var = 0.0;
  const double a = I.mark_p[0], g = I.mark_p[1];
  const double kappa = std::exp(a + 0.5 * g * g) - 1.0;
  // the jump regressor is carried divided by its compensator rate, so it
  // needs E[J] != 0; an asset that never jumps gets rate 0 (regressor 0)
  if (I.rate > 0.f && I.mark == SDEMC_MARK_LOGNORMAL && std::fabs(kappa) > 1e-9) {
    for (int i = 0; i < d; ++i) {
      double p = 1.0;
      if (I.jump_target == SDEMC_JUMP_ONE_ASSET) {
        const double lo = i > 0 ? I.jump_cdf[i - 1] : 0.0, hi = i < d - 1 ? I.jump_cdf[i] : 1.0;
        p = hi - lo;
      }
      cw.comp[i] = (float)((double)I.rate * p * kappa);
    }
    cw.jumps = 1;
    // E[J^2] for J = exp(N(a, g^2)) - 1
    cw.comp_j2 = (float)((double)I.rate * (std::exp(2.0 * a + 2.0 * g * g) - 2.0 * std::exp(a + 0.5 * g * g) + 1.0));
    jump_var = (double)I.rate * (a * a + g * g) / (I.jump_target == SDEMC_JUMP_ONE_ASSET ? d : 1);
  }
  switch (I.payoff) {
    case SDEMC_PAYOFF_EUROCALL: cw.wkind = 1; cw.agg = 0; break;
    case SDEMC_PAYOFF_EUROPUT: cw.wkind = 2; cw.agg = 0; break;
    case SDEMC_PAYOFF_BASKET_ARITH:
    case SDEMC_PAYOFF_BASKET_GEO: cw.wkind = 1; cw.agg = 1; break;
    case SDEMC_PAYOFF_RAINBOW:
    case SDEMC_PAYOFF_BESTOF: cw.wkind = 1; cw.agg = 2; break;
    default: cw.wkind = 0; break;
  }
  if (I.payoff_log || !(I.strike > 0.f)) cw.wkind = 0;
  // correlation from the packed Cholesky rows, then the underlying's variance
  double L[SDEMC_MAX_DIM][SDEMC_MAX_DIM] = {};
  for (int i = 0, q = 0; i < d; ++i)
    for (int j = 0; j <= i; ++j) L[i][j] = I.chol[q++];
  double sig[SDEMC_MAX_DIM];
  for (int i = 0; i < d; ++i) sig[i] = std::fabs((double)I.diff_q[i]);
  // Heston's price volatility is sqrt(v): weight with the initial variance's
  if (I.model == SDEMC_MODEL_HESTON) sig[0] = std::sqrt(std::max((double)I.x0[1], 0.0));
  double var = 0.0;
  if (cw.agg == 0) {
    var = sig[0] * sig[0];
  } else if (cw.agg == 1) {
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) {
        double c = 0.0;
        for (int k = 0; k < d; ++k) c += L[i][k] * L[j][k];
        var += sig[i] * sig[j] * c;
      }
    var /= (double)d * d;
  } else {
    for (int i = 0; i < d; ++i) var += sig[i] * sig[i];
    var /= d;
  }
  var = std::max(var + jump_var, 1e-8);
  cw.inv_sig = (float)(1.0 / std::sqrt(var));
  cw.drift = (float)((double)I.disc_rate + 0.5 * var);
  cw.T = I.T;
  cw.scale_over_k = cw.wkind ? (float)((double)I.payoff_scale / (double)I.strike) : 1.f;
  for (int i = 0; i < SDEMC_MAX_DIM; ++i)
    cw.inv_comp[i] = cw.comp[i] != 0.f ? (float)(1.0 / (double)cw.comp[i]) : 0.f;
  cw.inv_comp_j2 = cw.comp_j2 != 0.f ? (float)(1.0 / (double)cw.comp_j2) : 0.f;
  return cw;
}

struct Server {
  sdemc_server_cfg cfg{};
  int threads = 256;
  int64_t part_cap = 0;  // doubles per tick buffer
  int64_t fixed_bytes = 0;
  ServeSlot* slots_d = nullptr;
  TickBuf buf[kTickBufs];
  // tick-end stamps: a ring longer than the ticks in flight, so the previous
  // tick's end is still recorded when a tick is processed
  static constexpr int kStamps = 2 * kTickBufs + 2;
  cudaEvent_t stamp[kStamps] = {};
  int64_t ticks_enqueued = 0;
  double end_prev_ms = 0.0, last_end_ms = 0.0;  // device timeline of processed ticks

  std::vector<HostSlot> hs;
  std::vector<int> free_slots;
  std::vector<ServeInstall> staged;  // slot writes waiting for the next tick
  uint64_t seq = 0;

  std::mutex mu;
  std::condition_variable cv_in, cv_out;
  std::deque<Pending> pending;
  std::deque<sdemc_result> results;
  bool stop = false;
  int fatal = SDEMC_OK;
  sdemc_server_stats st{};
  std::thread th;

  int init(const sdemc_server_cfg& c);
  void release();
  void loop();
  void admit_locked();
  bool plan(TickBuf& B);
  int enqueue(TickBuf& B, const TickBuf& prev);
  int process(TickBuf& B);
  void finish(HostSlot& h, int status, double mean, double se, int64_t main_paths);
  void fail_all(int status);
};

int Server::init(const sdemc_server_cfg& c) {
  cfg = c;
  if (cfg.max_slots < 1 || cfg.max_slots > 65536) return fail(SDEMC_EINVAL, "max_slots %d outside 1..65536", cfg.max_slots);
  if (cfg.block_threads == 0) cfg.block_threads = 256;
  if (cfg.block_threads < 32 || cfg.block_threads > 256 || cfg.block_threads % 32)
    return fail(SDEMC_EINVAL, "block_threads %d must be a multiple of 32 in [32, 256]", cfg.block_threads);
  threads = cfg.block_threads;
  if (cfg.tick_work <= 0) cfg.tick_work = (int64_t)1 << 33;
  if (cfg.slice_work <= 0) cfg.slice_work = (int64_t)1 << 27;  // 2,000 req/s basket stream: p50/p99 2.95/22.5 ms (2^28: 3.3/24.5, 2^26: 2.45/24.3)
  if (cfg.side_streams < 0 || cfg.side_streams > 16) return fail(SDEMC_EINVAL, "side_streams %d outside 0..16", cfg.side_streams);
  if (cfg.policy != SDEMC_SERVE_FIFO && cfg.policy != SDEMC_SERVE_SRPT) return fail(SDEMC_EINVAL, "unknown policy %d", cfg.policy);
  int rc = check_cuda(cudaSetDevice(cfg.device), "cudaSetDevice");
  if (rc) return rc;
  const int64_t ms = cfg.max_slots;
  fixed_bytes = ms * (int64_t)sizeof(ServeSlot) +
                kTickBufs * (ms * (int64_t)(sizeof(ServeEntry) + sizeof(ServeInstall) + sizeof(ServeDone)) +
                     kNumClassKeys * 8);
  const int64_t min_part = kTickBufs * (kMaxSlicePaths / kChunk) * kServeMaxW * 8;
  if (cfg.mem_budget < fixed_bytes + min_part)
    return fail(SDEMC_ENOMEM, "mem_budget %lld below the %lld bytes of slot tables and one full slice",
                (long long)cfg.mem_budget, (long long)(fixed_bytes + min_part));
  int64_t share = (cfg.mem_budget - fixed_bytes) / kTickBufs;
  if (share > ((int64_t)1 << 30)) share = (int64_t)1 << 30;
  part_cap = share / 8;
  if ((rc = check_cuda(cudaMalloc(&slots_d, ms * sizeof(ServeSlot)), "slot table"))) return rc;
  for (int i = 0; i < kStamps; ++i)
    if ((rc = check_cuda(cudaEventCreate(&stamp[i]), "event create"))) return rc;
  for (TickBuf& B : buf) {
    if ((rc = check_cuda(cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking), "stream create"))) return rc;
    B.side.resize(cfg.side_streams);
    B.join.resize(cfg.side_streams);
    for (int i = 0; i < cfg.side_streams; ++i) {
      if ((rc = check_cuda(cudaStreamCreateWithFlags(&B.side[i], cudaStreamNonBlocking), "stream create"))) return rc;
      if ((rc = check_cuda(cudaEventCreateWithFlags(&B.join[i], cudaEventDisableTiming), "event create"))) return rc;
    }
    if ((rc = check_cuda(cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming), "event create"))) return rc;
    if ((rc = check_cuda(cudaEventCreateWithFlags(&B.red_done, cudaEventDisableTiming), "event create"))) return rc;
    if ((rc = check_cuda(cudaMallocHost(&B.entries_h, ms * sizeof(ServeEntry)), "pinned entries"))) return rc;
    if ((rc = check_cuda(cudaMallocHost(&B.installs_h, ms * sizeof(ServeInstall)), "pinned installs"))) return rc;
    if ((rc = check_cuda(cudaMallocHost(&B.done_h, ms * sizeof(ServeDone)), "pinned done"))) return rc;
    if ((rc = check_cuda(cudaMalloc(&B.entries_d, ms * sizeof(ServeEntry)), "entries"))) return rc;
    if ((rc = check_cuda(cudaMalloc(&B.installs_d, ms * sizeof(ServeInstall)), "installs"))) return rc;
    if ((rc = check_cuda(cudaMalloc(&B.done_d, ms * sizeof(ServeDone)), "done"))) return rc;
    if ((rc = check_cuda(cudaMalloc(&B.counters_d, kNumClassKeys * 8), "counters"))) return rc;
    if ((rc = check_cuda(cudaMalloc(&B.part_d, part_cap * 8), "tick partials"))) return rc;
    if ((rc = check_cuda(cudaEventCreate(&B.t0), "event create"))) return rc;
  }
  hs.assign(ms, HostSlot());
  free_slots.clear();
  for (int i = (int)ms - 1; i >= 0; --i) free_slots.push_back(i);
  st.mem_in_use = fixed_bytes;
  st.mem_peak = fixed_bytes;
  th = std::thread([this] { loop(); });
  return SDEMC_OK;
}

void Server::release() {
  for (TickBuf& B : buf) {
    if (B.stream) cudaStreamSynchronize(B.stream);
    for (cudaStream_t s : B.side) if (s) cudaStreamSynchronize(s);
  }
  for (TickBuf& B : buf) {
    for (cudaEvent_t e : B.join) if (e) cudaEventDestroy(e);
    if (B.fork) cudaEventDestroy(B.fork);
    if (B.red_done) cudaEventDestroy(B.red_done);
    for (cudaStream_t s : B.side) if (s) cudaStreamDestroy(s);
    if (B.stream) cudaStreamDestroy(B.stream);
    if (B.entries_h) cudaFreeHost(B.entries_h);
    if (B.installs_h) cudaFreeHost(B.installs_h);
    if (B.done_h) cudaFreeHost(B.done_h);
    if (B.entries_d) cudaFree(B.entries_d);
    if (B.installs_d) cudaFree(B.installs_d);
    if (B.done_d) cudaFree(B.done_d);
    if (B.counters_d) cudaFree(B.counters_d);
    if (B.part_d) cudaFree(B.part_d);
    if (B.t0) cudaEventDestroy(B.t0);
    B = TickBuf();
  }
  if (slots_d) cudaFree(slots_d);
  slots_d = nullptr;
  for (cudaEvent_t& e : stamp) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
}

// Pending requests -> free slots, in arrival order, while the budget allows.
void Server::admit_locked() {
  while (!pending.empty() && !free_slots.empty()) {
    const Pending& P = pending.front();
    const sdemc_inst& I = P.req.inst;
    const bool lcv = P.req.estimator == SDEMC_EST_LINEAR_CV && lcv_supported(I);
    const double cost = path_cost(I);
    int64_t slice = (int64_t)std::ceil((double)cfg.slice_work / std::max(cost, 1.0));
    slice = std::min(std::max(slice, kMinSlicePaths), kMaxSlicePaths);
    slice = (slice + kChunk - 1) / kChunk * kChunk;
    const int wmax = lcv ? pilot_width(I.dim) : 3;
    const int64_t reserve = (int64_t)sizeof(ServeSlot) + kTickBufs * (slice / kChunk) * wmax * 8;
    if (st.mem_in_use + reserve > cfg.mem_budget) break;
    const int s = free_slots.back();
    free_slots.pop_back();
    HostSlot& h = hs[s];
    h = HostSlot();
    h.used = true;
    h.req = P.req;
    h.t_arrive = P.t_arrive;
    h.t_admit = now_ns();
    h.seq = seq++;
    h.phase = 0;
    h.kind = lcv ? kKindPilotStats : kKindPlain;
    h.width = kind_width(h.kind, I.dim);
    h.est = lcv ? SDEMC_EST_LINEAR_CV : SDEMC_EST_PLAIN;
    h.cursor = 0;
    h.phase_end = I.num_paths;
    h.pilot_paths = I.num_paths;
    h.slice = slice;
    h.cost = cost;
    h.reserve = reserve;
    st.mem_in_use += reserve;
    st.mem_peak = std::max(st.mem_peak, st.mem_in_use);
    st.admitted++;
    st.active++;
    ServeInstall in{};
    in.slot = s;
    in.whole = 1;
    in.rec.inst = I;
    in.rec.st.cursor = 0;
    in.rec.st.phase_end = h.phase_end;
    in.rec.st.phase = 0;
    in.rec.st.width = h.width;
    in.rec.st.kind = h.kind;
    h.cw = serve_cv_weights(I);
    in.rec.st.cw = h.cw;
    staged.push_back(in);
    pending.pop_front();
  }
  st.pending = (int64_t)pending.size();
}

bool Server::plan(TickBuf& B) {
  std::vector<int> cand;
  for (int s = 0; s < (int)hs.size(); ++s) {
    const HostSlot& h = hs[s];
    if (h.used && !h.awaiting && h.cursor < h.phase_end) cand.push_back(s);
  }
  if (cfg.policy == SDEMC_SERVE_SRPT) {
    std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) {
      const double ra = (double)(hs[a].phase_end - hs[a].cursor) * hs[a].cost;
      const double rb = (double)(hs[b].phase_end - hs[b].cursor) * hs[b].cost;
      return ra < rb || (ra == rb && hs[a].seq < hs[b].seq);
    });
  } else {
    std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) { return hs[a].seq < hs[b].seq; });
  }
  struct Pick { int key, slot; int64_t nch; };
  std::vector<Pick> picks;
  double work = 0.0;
  int64_t part = 0;
  int ndone = 0;
  B.path_steps = 0.0;
  for (int s : cand) {
    HostSlot& h = hs[s];
    const int64_t n = std::min(h.slice, h.phase_end - h.cursor);
    const int64_t nch = (n + kChunk - 1) / kChunk;
    const double w = (double)n * h.cost;
    if (!picks.empty() && work + w > (double)cfg.tick_work) break;
    if (part + nch * h.width > part_cap) break;
    work += w;
    part += nch * h.width;
    B.path_steps += w / (double)h.req.inst.dim;
    picks.push_back({class_key(h.kind, h.req.inst), s, nch});
  }
  if (picks.empty() && staged.empty()) return false;
  std::stable_sort(picks.begin(), picks.end(), [](const Pick& a, const Pick& b) { return a.key < b.key; });
  int64_t chunk = 0, poff = 0;
  for (size_t i = 0; i < picks.size(); ++i) {
    HostSlot& h = hs[picks[i].slot];
    ServeEntry& E = B.entries_h[i];
    E.slot = picks[i].slot;
    E.width = h.width;
    E.kind = h.kind;
    E.chunk_begin = chunk;
    E.nchunks = picks[i].nch;
    E.part_off = poff;
    E.base = h.cursor;
    E.end = h.phase_end;
    chunk += E.nchunks;
    poff += E.nchunks * E.width;
    h.cursor = std::min(h.cursor + E.nchunks * kChunk, h.phase_end);
    if (h.cursor == h.phase_end) {
      E.done = ndone++;
      h.awaiting = true;
    } else {
      E.done = -1;
    }
  }
  B.n_entries = (int)picks.size();
  B.n_done = ndone;
  B.n_installs = (int)staged.size();
  std::copy(staged.begin(), staged.end(), B.installs_h);
  staged.clear();
  return true;
}

int Server::enqueue(TickBuf& B, const TickBuf& prev) {
  int rc;
  cudaStream_t stream = B.stream;
  B.seq = ticks_enqueued++;
  if ((rc = check_cuda(cudaEventRecord(B.t0, stream), "tick start"))) return rc;
  if (B.n_installs > 0 &&
      (rc = check_cuda(cudaMemcpyAsync(B.installs_d, B.installs_h, B.n_installs * sizeof(ServeInstall),
                                       cudaMemcpyHostToDevice, stream), "installs upload")))
    return rc;
  if (B.n_entries > 0 &&
      (rc = check_cuda(cudaMemcpyAsync(B.entries_d, B.entries_h, B.n_entries * sizeof(ServeEntry),
                                       cudaMemcpyHostToDevice, stream), "plan upload")))
    return rc;
  // installs touch only slots that no tick in flight has entries for (new
  // requests, and slots whose previous phase ended in a tick already processed)
  if ((rc = launch_serve_install(slots_d, B.installs_d, B.n_installs, B.counters_d, kNumClassKeys, stream)))
    return rc;
  const int nside = (int)B.side.size();
  if (nside > 0) {
    if ((rc = check_cuda(cudaEventRecord(B.fork, stream), "fork record"))) return rc;
    for (int j = 0; j < nside; ++j)
      if ((rc = check_cuda(cudaStreamWaitEvent(B.side[j], B.fork, 0), "fork wait"))) return rc;
  }
  int k = 0, launched = 0;
  while (k < B.n_entries && rc == SDEMC_OK) {
    const ServeEntry& E0 = B.entries_h[k];
    const sdemc_inst& I = hs[E0.slot].req.inst;
    const int key = class_key(E0.kind, I);
    int j = k + 1;
    while (j < B.n_entries && class_key(B.entries_h[j].kind, hs[B.entries_h[j].slot].req.inst) == key) ++j;
    ServeParams P;
    P.slots = slots_d;
    P.entries = B.entries_d;
    P.first = k;
    P.count = j - k;
    P.chunk_begin = B.entries_h[k].chunk_begin;
    P.chunk_end = B.entries_h[j - 1].chunk_begin + B.entries_h[j - 1].nchunks;
    P.counter = B.counters_d + key;
    P.part = B.part_d;
    P.uniform_seed = 1;
    for (int e = k + 1; e < j; ++e)
      if (hs[B.entries_h[e].slot].req.inst.seed != I.seed) P.uniform_seed = 0;
    P.rk = make_round_keys(I.seed);
    const int64_t chunks = P.chunk_end - P.chunk_begin;
    cudaStream_t ks = nside > 0 ? B.side[launched % nside] : stream;
    if (E0.kind == kKindPlain)
      rc = launch_serve_plain(I.dim, I.noise, loop_mode_of(I), P, threads, chunks, ks);
    else
      rc = launch_serve_cv(E0.kind, I.dim, P, threads, chunks, ks);
    ++launched;
    k = j;
  }
  B.launches = launched + 1 + (B.n_entries > 0 ? 1 : 0);
  // join the side streams back even after a failed launch
  for (int j = 0; j < nside; ++j) {
    int jr = check_cuda(cudaEventRecord(B.join[j], B.side[j]), "join record");
    if (jr == SDEMC_OK) jr = check_cuda(cudaStreamWaitEvent(stream, B.join[j], 0), "join wait");
    if (rc == SDEMC_OK) rc = jr;
  }
  if (rc) return rc;
  // each slot's sums are folded tick after tick: this reduction follows the
  // previous tick's (a never-recorded event is already complete)
  if ((rc = check_cuda(cudaStreamWaitEvent(stream, prev.red_done, 0), "reduce order"))) return rc;
  if ((rc = launch_serve_reduce(slots_d, B.entries_d, B.n_entries, B.part_d, B.done_d, stream))) return rc;
  if ((rc = check_cuda(cudaEventRecord(B.red_done, stream), "reduce done"))) return rc;
  if (B.n_done > 0 &&
      (rc = check_cuda(cudaMemcpyAsync(B.done_h, B.done_d, B.n_done * sizeof(ServeDone), cudaMemcpyDeviceToHost,
                                       stream), "done readback")))
    return rc;
  return check_cuda(cudaEventRecord(stamp[B.seq % kStamps], stream), "tick end");
}

void Server::finish(HostSlot& h, int status, double mean, double se, int64_t main_paths) {
  sdemc_result r{};
  r.tag = h.req.tag;
  r.status = status;
  r.estimator = h.est;
  r.mean = mean;
  r.se = se;
  r.pilot_mean = h.pilot_mean;
  r.pilot_se = h.pilot_se;
  r.vrf = h.vrf;
  r.pilot_paths = h.pilot_paths;
  r.main_paths = main_paths;
  r.t_arrive_ns = h.t_arrive;
  r.t_admit_ns = h.t_admit;
  r.t_done_ns = now_ns();
  for (int i = 0; i < kServeMaxR; ++i) r.beta[i] = h.beta[i];
  const int s = (int)(&h - hs.data());
  {
    std::lock_guard<std::mutex> lk(mu);
    results.push_back(r);
    st.completed++;
    st.active--;
    st.mem_in_use -= h.reserve;
    free_slots.push_back(s);
  }
  h.used = false;
  cv_out.notify_all();
}

int Server::process(TickBuf& B) {
  cudaEvent_t t_end = stamp[B.seq % kStamps];
  int rc = check_cuda(cudaEventSynchronize(t_end), "tick wait");
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, B.t0, t_end);
  // place the tick on one device timeline: its end relative to the previous
  // processed tick's end (both stamps still recorded: the ring outlives the
  // ticks in flight), its start by its own duration; busy time is the
  // union of the tick intervals (ticks overlap)
  double end_ms = 0.0;
  if (B.seq > 0) {
    float gap = 0.f;
    cudaEventElapsedTime(&gap, stamp[(B.seq - 1) % kStamps], t_end);
    end_ms = end_prev_ms + (double)gap;
  }
  const double start_ms = end_ms - (double)ms;
  const double added = std::max(0.0, end_ms - std::max(start_ms, B.seq > 0 ? last_end_ms : start_ms));
  end_prev_ms = end_ms;
  last_end_ms = B.seq > 0 ? std::max(last_end_ms, end_ms) : end_ms;
  {
    std::lock_guard<std::mutex> lk(mu);
    st.ticks++;
    st.busy_s += added * 1e-3;
    int b = 0;
    for (double edge = 0.125; b < 15 && ms >= edge; edge *= 2.0) ++b;
    st.tick_hist[b]++;
    st.path_steps += (int64_t)B.path_steps;
    st.launches += B.launches;
    st.h2d_bytes += (int64_t)B.n_installs * (int64_t)sizeof(ServeInstall) +
                    (int64_t)B.n_entries * (int64_t)sizeof(ServeEntry);
    st.d2h_bytes += (int64_t)B.n_done * (int64_t)sizeof(ServeDone);
  }
  for (int i = 0; i < B.n_done; ++i) {
    const ServeDone& R = B.done_h[i];
    HostSlot& h = hs[R.slot];
    h.awaiting = false;
    const double n = R.acc[2];
    const double mean = n > 0 ? R.acc[0] / n : 0.0;
    const double var = n > 1 ? std::max((R.acc[1] - R.acc[0] * R.acc[0] / n) / (n - 1.0), 0.0) : 0.0;
    if (R.status != SDEMC_OK) {
      finish(h, R.status, mean, std::sqrt(var / std::max(n, 1.0)), h.phase == 1 ? (int64_t)n : 0);
      continue;
    }
    if (h.phase == 1) {
      finish(h, SDEMC_OK, mean, std::sqrt(var / std::max(n, 1.0)), (int64_t)n);
      continue;
    }
    // pilot finished: size the main run
    h.pilot_mean = mean;
    h.pilot_se = std::sqrt(var / std::max(n, 1.0));
    double var_main = var;
    int kind = kKindPlain;
    h.est = SDEMC_EST_PLAIN;
    h.vrf = 1.0;
    for (int k = 0; k < kServeMaxR; ++k) h.beta[k] = 0.f;
    if (h.kind == kKindPilotStats && n > 2) {
      const int nr = num_regressors(h.req.inst.dim);
      double ybar[kServeMaxR], C[kServeMaxR * kServeMaxR], c[kServeMaxR], beta[kServeMaxR];
      for (int a = 0; a < nr; ++a) ybar[a] = R.acc[3 + a] / n;
      int q = 3 + nr;
      for (int a = 0; a < nr; ++a)
        for (int b = a; b < nr; ++b, ++q) {
          const double v = (R.acc[q] - n * ybar[a] * ybar[b]) / (n - 1.0);
          C[a * nr + b] = v;
          C[b * nr + a] = v;
        }
      for (int a = 0; a < nr; ++a) c[a] = (R.acc[q + a] - n * ybar[a] * mean) / (n - 1.0);
      if (solve_spd(nr, C, c, beta)) {
        double explained = 0.0;
        for (int a = 0; a < nr; ++a) explained += beta[a] * c[a];
        const double resid = var - explained;
        // keep the control variate only when it pays: 5% less variance
        if (resid > 0.0 && resid < var / 1.05) {
          var_main = resid;
          kind = kKindLcv;
          h.est = SDEMC_EST_LINEAR_CV;
          h.vrf = var / resid;
          for (int a = 0; a < nr; ++a) h.beta[a] = (float)beta[a];
        }
      }
    }
    const double eps = h.req.rel_target * std::fabs(mean);
    int64_t nmain;
    if (var_main <= 0.0) {
      finish(h, SDEMC_OK, mean, 0.0, 0);  // a deterministic payoff: the pilot is exact
      continue;
    }
    const int64_t cap = h.req.max_paths > 0 ? h.req.max_paths : ((int64_t)1 << 36);
    if (eps > 0.0 && std::isfinite(eps)) {
      const double want = std::ceil(kZ95 * kZ95 * var_main / (eps * eps));
      nmain = want >= (double)cap ? cap : (int64_t)want;
    } else {
      nmain = cap;
    }
    nmain = std::max<int64_t>(nmain, 64);
    h.phase = 1;
    h.kind = kind;
    h.width = 3;
    h.phase_end = h.cursor + nmain;
    ServeInstall in{};
    in.slot = R.slot;
    in.whole = 0;
    for (int k = 0; k < kServeMaxR; ++k) in.rec.st.beta[k] = h.beta[k];
    in.rec.st.cw = h.cw;
    in.rec.st.cursor = h.cursor;
    in.rec.st.phase_end = h.phase_end;
    in.rec.st.phase = 1;
    in.rec.st.width = 3;
    in.rec.st.status = 0;
    in.rec.st.kind = kind;
    staged.push_back(in);
  }
  return SDEMC_OK;
}

void Server::fail_all(int status) {
  std::lock_guard<std::mutex> lk(mu);
  fatal = status;
  for (HostSlot& h : hs) {
    if (!h.used) continue;
    sdemc_result r{};
    r.tag = h.req.tag;
    r.status = status;
    r.t_arrive_ns = h.t_arrive;
    r.t_admit_ns = h.t_admit;
    r.t_done_ns = now_ns();
    results.push_back(r);
    h.used = false;
  }
  for (const Pending& p : pending) {
    sdemc_result r{};
    r.tag = p.req.tag;
    r.status = status;
    r.t_arrive_ns = p.t_arrive;
    r.t_done_ns = now_ns();
    results.push_back(r);
  }
  pending.clear();
  cv_out.notify_all();
}

void Server::loop() {
  if (cudaSetDevice(cfg.device) != cudaSuccess) {
    fail_all(SDEMC_ECUDA);
    return;
  }
  // buffers in flight: oldest, oldest + 1, ... (count of them), in tick order
  int oldest = 0, count = 0;
  for (;;) {
    {
      std::lock_guard<std::mutex> lk(mu);
      if (stop) break;
      admit_locked();
    }
    bool launched = false;
    if (count < kTickBufs) {
      const int next = (oldest + count) % kTickBufs;
      TickBuf& B = buf[next];
      if (plan(B)) {
        if (enqueue(B, buf[(next + kTickBufs - 1) % kTickBufs]) != SDEMC_OK) {
          fail_all(SDEMC_ECUDA);
          break;
        }
        launched = true;
        ++count;
      }
    }
    // handle finished ticks in order; block on the oldest only when every
    // buffer is in flight or there was nothing new to launch
    bool failed = false;
    while (count > 0) {
      const cudaError_t q = cudaEventQuery(stamp[buf[oldest].seq % kStamps]);
      if (q == cudaErrorNotReady) (void)cudaGetLastError();  // not an error: the tick still runs
      const bool done = q == cudaSuccess;
      if (!done && launched && count < kTickBufs) break;
      if (process(buf[oldest]) != SDEMC_OK) {
        failed = true;
        break;
      }
      oldest = (oldest + 1) % kTickBufs;
      --count;
      if (!done) break;  // waited once: plan again before waiting more
    }
    if (failed) {
      fail_all(SDEMC_ECUDA);
      break;
    }
    if (launched || count > 0) continue;
    if (!staged.empty()) continue;
    std::unique_lock<std::mutex> lk(mu);
    if (stop) break;
    bool runnable = false;
    for (const HostSlot& h : hs)
      if (h.used && !h.awaiting && h.cursor < h.phase_end) { runnable = true; break; }
    // idle: sleep until a request arrives (admission runs at the top)
    if (!runnable) cv_in.wait_for(lk, std::chrono::milliseconds(2));
  }
  for (int i = 0; i < count; ++i) cudaEventSynchronize(stamp[buf[(oldest + i) % kTickBufs].seq % kStamps]);
}

}  // namespace sdemc

using namespace sdemc;

struct sdemc_server {
  Server* impl;
};

extern "C" int sdemc_server_create(const sdemc_server_cfg* cfg, sdemc_server** out) {
  if (!cfg || !out) return fail(SDEMC_EINVAL, "null server argument");
  *out = nullptr;
  Server* S = new (std::nothrow) Server();
  if (!S) return fail(SDEMC_ENOMEM, "server allocation");
  const int rc = S->init(*cfg);
  if (rc) {
    if (S->th.joinable()) {
      { std::lock_guard<std::mutex> lk(S->mu); S->stop = true; }
      S->cv_in.notify_all();
      S->th.join();
    }
    S->release();
    delete S;
    return rc;
  }
  sdemc_server* h = new (std::nothrow) sdemc_server{S};
  if (!h) {
    { std::lock_guard<std::mutex> lk(S->mu); S->stop = true; }
    S->cv_in.notify_all();
    S->th.join();
    S->release();
    delete S;
    return fail(SDEMC_ENOMEM, "server handle allocation");
  }
  *out = h;
  return SDEMC_OK;
}

extern "C" int sdemc_server_admit(sdemc_server* srv, const sdemc_request* req) {
  if (!srv || !srv->impl || !req) return fail(SDEMC_EINVAL, "null server argument");
  Server& S = *srv->impl;
  int rc = validate_inst(&req->inst);
  if (rc) return rc;
  if (req->inst.num_paths < 2) return fail(SDEMC_EINVAL, "pilot needs at least 2 paths");
  if (!(req->rel_target > 0.0) || !std::isfinite(req->rel_target))
    return fail(SDEMC_EINVAL, "rel_target must be positive");
  if (req->estimator != SDEMC_EST_PLAIN && req->estimator != SDEMC_EST_LINEAR_CV)
    return fail(SDEMC_EINVAL, "unknown estimator %d", req->estimator);
  if (req->max_paths < 0) return fail(SDEMC_EINVAL, "max_paths must be >= 0");
  const int64_t worst = (int64_t)sizeof(ServeSlot) + 2 * (kMaxSlicePaths / kChunk) * pilot_width(req->inst.dim) * 8;
  if (S.fixed_bytes + worst > S.cfg.mem_budget)
    return fail(SDEMC_ENOMEM, "request can never fit the server's memory budget");
  {
    std::lock_guard<std::mutex> lk(S.mu);
    if (S.fatal) return fail(S.fatal, "server stopped after a device error");
    if (S.stop) return fail(SDEMC_EINVAL, "server is shutting down");
    S.pending.push_back({*req, now_ns()});
    S.st.submitted++;
    S.st.pending = (int64_t)S.pending.size();
  }
  S.cv_in.notify_all();
  return SDEMC_OK;
}

extern "C" int sdemc_server_poll(sdemc_server* srv, sdemc_result* out, int max, int* n_out, int64_t wait_ns) {
  if (!srv || !srv->impl || !n_out || max < 0 || (max > 0 && !out)) return fail(SDEMC_EINVAL, "bad poll arguments");
  Server& S = *srv->impl;
  std::unique_lock<std::mutex> lk(S.mu);
  if (S.results.empty() && wait_ns > 0)
    S.cv_out.wait_for(lk, std::chrono::nanoseconds(wait_ns), [&] { return !S.results.empty(); });
  int n = 0;
  while (n < max && !S.results.empty()) {
    out[n++] = S.results.front();
    S.results.pop_front();
  }
  *n_out = n;
  return SDEMC_OK;
}

extern "C" int sdemc_server_stats_get(sdemc_server* srv, sdemc_server_stats* out) {
  if (!srv || !srv->impl || !out) return fail(SDEMC_EINVAL, "null server argument");
  std::lock_guard<std::mutex> lk(srv->impl->mu);
  *out = srv->impl->st;
  return SDEMC_OK;
}

extern "C" int sdemc_server_destroy(sdemc_server* srv) {
  if (!srv) return SDEMC_OK;
  Server* S = srv->impl;
  if (S) {
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->stop = true;
    }
    S->cv_in.notify_all();
    if (S->th.joinable()) S->th.join();
    S->release();
    delete S;
  }
  delete srv;
  return SDEMC_OK;
}

extern "C" int sdemc_serve_sizes(size_t* out, int n) {
  if (!out || n < 4) return fail(SDEMC_EINVAL, "need room for 4 sizes");
  out[0] = sizeof(sdemc_server_cfg);
  out[1] = sizeof(sdemc_request);
  out[2] = sizeof(sdemc_result);
  out[3] = sizeof(sdemc_server_stats);
  return SDEMC_OK;
}
