// k_batch.cu — K8: many heterogeneous pricing instances in one pass.
//
// A batch is planned on the host (sdemc_batch_plan): instances are grouped
// into classes of equal (dim, noise layout, loop variant) so each class runs a
// kernel compiled for its dimension, ordered by descending cost per chunk,
// and laid out as one run of 32-path chunks per class.  Each class kernel is
// persistent: a warp takes the next chunk from the class counter, finds its
// instance by binary search on the chunk prefix, stages that descriptor and
// its Philox round keys in shared memory, and runs exactly the per-path code
// of the single-instance kernel (simulate + payoff + warp butterfly).  The
// batched FP64 reduction then sums each instance's chunks in the same fixed
// order as K10, so every instance's result is bit-identical to pricing it
// alone — the property the serving layer relies on.
#include "k_batch_kern.cuh"

namespace sdemc {

struct BatchReduceParams {
  const int64_t* chunk_prefix;
  const int64_t* group_prefix;
  const int32_t* order;
  int n;
  const double* part;
  double* groups;
  int32_t* status;
  unsigned* counters;
  double* out;
};

// K10 per instance, all instances in one launch (CTA = one reduction group).
__global__ void __launch_bounds__(kGroup) batch_reduce_kernel(const __grid_constant__ BatchReduceParams R) {
  __shared__ double sh[3][kGroup];
  __shared__ bool last;
  __shared__ int s_inst;
  const int t = threadIdx.x;
  const int64_t g = blockIdx.x;
  if (t == 0) {
    int a = 0, b = R.n;  // group_prefix[a] <= g < group_prefix[b]
    while (b - a > 1) {
      const int m = (a + b) >> 1;
      if (R.group_prefix[m] <= g) a = m; else b = m;
    }
    s_inst = a;
  }
  __syncthreads();
  const int i = s_inst;
  const int64_t cbase = R.chunk_prefix[i], nch = R.chunk_prefix[i + 1] - cbase;
  const int64_t gbase = R.group_prefix[i], ngroups = R.group_prefix[i + 1] - gbase;
  const int64_t c = (g - gbase) * kGroup + t;
#pragma unroll
  for (int w = 0; w < 3; ++w) sh[w][t] = c < nch ? R.part[(cbase + c) * 3 + w] : 0.0;
  __syncthreads();
  for (int o = kGroup / 2; o > 0; o >>= 1) {
    if (t < o)
      for (int w = 0; w < 3; ++w) sh[w][t] += sh[w][t + o];
    __syncthreads();
  }
  if (t == 0) {
    for (int w = 0; w < 3; ++w) R.groups[g * 3 + w] = sh[w][0];
    __threadfence();
    last = atomicAdd(&R.counters[i], 1u) == (unsigned)(ngroups - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[3] = {0.0, 0.0, 0.0};
  for (int64_t q = t; q < ngroups; q += kGroup)
    for (int w = 0; w < 3; ++w) acc[w] += __ldcg(&R.groups[(gbase + q) * 3 + w]);
  __syncthreads();
  for (int w = 0; w < 3; ++w) sh[w][t] = acc[w];
  __syncthreads();
  for (int o = kGroup / 2; o > 0; o >>= 1) {
    if (t < o)
      for (int w = 0; w < 3; ++w) sh[w][t] += sh[w][t + o];
    __syncthreads();
  }
  if (t == 0) {
    const double s = sh[0][0], s2 = sh[1][0], n = sh[2][0];
    double* o = R.out + (size_t)R.order[i] * 6;
    o[0] = s; o[1] = s2; o[2] = n;
    o[3] = n > 0 ? s / n : 0.0;
    o[4] = n > 1 ? (s2 - s * s / n) / (n - 1.0) : 0.0;
    o[5] = (double)R.status[i];
    R.status[i] = 0;
    R.counters[i] = 0u;
  }
}

// ----------------------------------------------------------- host side ----
static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct PlanLayout {
  size_t classes, insts, order, chunk_prefix, group_prefix, total;
};

static PlanLayout plan_layout(int n) {
  PlanLayout L;
  size_t off = align_up(sizeof(sdemc_batch_header), 256);
  L.classes = off; off = align_up(off + (size_t)(n > 0 ? n : 1) * sizeof(sdemc_batch_class), 256);
  L.insts = off;   off = align_up(off + (size_t)n * sizeof(sdemc_inst), 256);
  L.order = off;   off = align_up(off + (size_t)n * sizeof(int32_t), 256);
  L.chunk_prefix = off; off = align_up(off + (size_t)(n + 1) * sizeof(int64_t), 256);
  L.group_prefix = off; off = align_up(off + (size_t)(n + 1) * sizeof(int64_t), 256);
  L.total = off;
  return L;
}

struct ScratchLayout {
  size_t counters, status, red_counters, part, groups, total;
};

static ScratchLayout scratch_layout(const sdemc_batch_header& H) {
  ScratchLayout S;
  size_t off = 0;
  S.counters = off; off = align_up(off + (size_t)(H.n_class > 0 ? H.n_class : 1) * 8, 256);
  S.status = off; off = align_up(off + (size_t)(H.n_inst > 0 ? H.n_inst : 1) * 4, 256);
  S.red_counters = off; off = align_up(off + (size_t)(H.n_inst > 0 ? H.n_inst : 1) * 4, 256);
  S.part = off; off = align_up(off + (size_t)H.total_chunks * 3 * 8, 256);
  S.groups = off; off = align_up(off + (size_t)H.total_groups * 3 * 8, 256);
  S.total = off;
  return S;
}

static int loop_mode(const sdemc_inst& I) {
  return (I.flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP) ? kModeNominal : 0;
}

static int launch_class(int dim, int noise, int mode, const BatchParams& B, const sdemc_cfg* cfg,
                        int64_t chunks, cudaStream_t s) {
  int rc = SDEMC_OK;
  switch (noise) {
    case SDEMC_NOISE_DIAG: rc = launch_batch_noise<SDEMC_NOISE_DIAG>(dim, mode, B, cfg, chunks, s); break;
    case SDEMC_NOISE_INDEP_SHARED:
      rc = launch_batch_noise<SDEMC_NOISE_INDEP_SHARED>(dim, mode, B, cfg, chunks, s);
      break;
    case SDEMC_NOISE_INDEP_PAIR: rc = launch_batch_noise<SDEMC_NOISE_INDEP_PAIR>(dim, mode, B, cfg, chunks, s); break;
    default: return fail(SDEMC_EINVAL, "noise layout %d unknown", noise);
  }
  return rc;
}

// Fork/join events for class kernels on side streams (one set per device).
struct EventPool {
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[64] = {};
};
static EventPool g_events[64];

static int events_for_device(EventPool** out) {
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= 64) return fail(SDEMC_EINVAL, "device %d out of range", dev);
  EventPool& P = g_events[dev];
  if (!P.fork) {
    if ((rc = check_cuda(cudaEventCreateWithFlags(&P.fork, cudaEventDisableTiming), "event create"))) return rc;
    for (int i = 0; i < 64; ++i)
      if ((rc = check_cuda(cudaEventCreateWithFlags(&P.join[i], cudaEventDisableTiming), "event create"))) return rc;
  }
  *out = &P;
  return SDEMC_OK;
}

}  // namespace sdemc

using namespace sdemc;

extern "C" size_t sdemc_batch_plan_bytes(int n) { return n < 0 ? 0 : plan_layout(n).total; }

extern "C" int sdemc_batch_plan(const sdemc_inst* h_insts, int n, void* h_blob, size_t blob_bytes) {
  if (n < 0 || (n > 0 && !h_insts) || !h_blob) return fail(SDEMC_EINVAL, "bad batch plan arguments");
  const PlanLayout L = plan_layout(n);
  if (blob_bytes < L.total) return fail(SDEMC_ENOMEM, "plan blob %zu bytes < required %zu", blob_bytes, L.total);
  for (int i = 0; i < n; ++i) {
    const int rc = validate_inst(&h_insts[i]);
    if (rc) return rc;
  }
  char* blob = static_cast<char*>(h_blob);
  memset(blob, 0, L.total);
  // order instances by class key, then by descending cost per chunk
  int32_t* order = reinterpret_cast<int32_t*>(blob + L.order);
  for (int i = 0; i < n; ++i) order[i] = i;
  auto key = [&](int i) {
    const sdemc_inst& I = h_insts[i];
    return (I.dim * 8 + I.noise) * 4 + loop_mode(I);
  };
  auto cost = [&](int i) {
    const sdemc_inst& I = h_insts[i];
    return (double)I.num_steps + (double)I.rate * (double)I.T;
  };
  // insertion-stable sort (n is at most a few thousand)
  for (int i = 1; i < n; ++i) {
    const int v = order[i];
    int j = i - 1;
    while (j >= 0 && (key(order[j]) > key(v) || (key(order[j]) == key(v) && cost(order[j]) < cost(v)))) {
      order[j + 1] = order[j];
      --j;
    }
    order[j + 1] = v;
  }
  sdemc_inst* insts = reinterpret_cast<sdemc_inst*>(blob + L.insts);
  int64_t* cp = reinterpret_cast<int64_t*>(blob + L.chunk_prefix);
  int64_t* gp = reinterpret_cast<int64_t*>(blob + L.group_prefix);
  sdemc_batch_class* cls = reinterpret_cast<sdemc_batch_class*>(blob + L.classes);
  int ncls = 0;
  cp[0] = 0;
  gp[0] = 0;
  for (int i = 0; i < n; ++i) {
    const sdemc_inst& I = h_insts[order[i]];
    insts[i] = I;
    const int64_t nch = num_chunks(&I);
    cp[i + 1] = cp[i] + nch;
    gp[i + 1] = gp[i] + num_groups_for(nch);
    if (i == 0 || key(order[i]) != key(order[i - 1])) {
      sdemc_batch_class& C = cls[ncls++];
      C.dim = I.dim; C.noise = I.noise; C.mode = loop_mode(I); C.count = 0; C.first = i;
      C.chunk_begin = cp[i];
    }
    sdemc_batch_class& C = cls[ncls - 1];
    C.count += 1;
    C.chunk_end = cp[i + 1];
  }
  sdemc_batch_header* H = reinterpret_cast<sdemc_batch_header*>(blob);
  H->n_inst = n;
  H->n_class = ncls;
  H->total_chunks = cp[n];
  H->total_groups = gp[n];
  H->off_classes = (int64_t)L.classes;
  H->off_insts = (int64_t)L.insts;
  H->off_order = (int64_t)L.order;
  H->off_chunk_prefix = (int64_t)L.chunk_prefix;
  H->off_group_prefix = (int64_t)L.group_prefix;
  return SDEMC_OK;
}

extern "C" size_t sdemc_batch_scratch_bytes(const void* h_blob) {
  if (!h_blob) return 0;
  return scratch_layout(*static_cast<const sdemc_batch_header*>(h_blob)).total;
}

extern "C" int sdemc_price_batch(const void* h_blob, const void* d_blob, void* d_scratch, size_t scratch_bytes,
                                 double* d_out, const sdemc_cfg* h_cfgs, void* const* side_streams, int n_side,
                                 void* stream) {
  if (!h_blob || !d_blob || !d_scratch || !d_out) return fail(SDEMC_EINVAL, "null batch argument");
  const sdemc_batch_header& H = *static_cast<const sdemc_batch_header*>(h_blob);
  if (H.n_inst < 0 || H.n_class < 0 || H.n_class > H.n_inst + 1) return fail(SDEMC_EINVAL, "corrupt batch plan");
  const ScratchLayout S = scratch_layout(H);
  if (scratch_bytes < S.total) return fail(SDEMC_ENOMEM, "batch scratch %zu < required %zu", scratch_bytes, S.total);
  if (n_side < 0 || n_side > 64 || (n_side > 0 && !side_streams)) return fail(SDEMC_EINVAL, "bad side streams");
  if (H.n_inst == 0) return SDEMC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const char* hb = static_cast<const char*>(h_blob);
  const char* db = static_cast<const char*>(d_blob);
  char* sc = static_cast<char*>(d_scratch);
  const sdemc_batch_class* cls = reinterpret_cast<const sdemc_batch_class*>(hb + H.off_classes);
  int rc = check_cuda(cudaMemsetAsync(sc, 0, S.part, s), "clear batch counters");
  if (rc) return rc;
  EventPool* ev = nullptr;
  int forked = 0;  // side streams that wait on the fork event and must be joined back
  if (n_side > 0) {
    if ((rc = events_for_device(&ev))) return rc;
    if ((rc = check_cuda(cudaEventRecord(ev->fork, s), "fork record"))) return rc;
    for (int j = 0; j < n_side && rc == SDEMC_OK; ++j) {
      rc = check_cuda(cudaStreamWaitEvent((cudaStream_t)side_streams[j], ev->fork, 0), "fork wait");
      if (rc == SDEMC_OK) ++forked;
    }
  }
  // a failure after the fork still joins every forked side stream back into
  // `stream` (under stream capture an unjoined fork invalidates the graph)
  for (int k = 0; k < H.n_class && rc == SDEMC_OK; ++k) {
    const sdemc_batch_class& C = cls[k];
    BatchParams B;
    B.insts = reinterpret_cast<const sdemc_inst*>(db + H.off_insts);
    B.chunk_prefix = reinterpret_cast<const int64_t*>(db + H.off_chunk_prefix);
    B.first = C.first;
    B.count = C.count;
    B.chunk_begin = C.chunk_begin;
    B.chunk_end = C.chunk_end;
    B.counter = reinterpret_cast<unsigned long long*>(sc + S.counters) + k;
    B.status = reinterpret_cast<int32_t*>(sc + S.status);
    B.part = reinterpret_cast<double*>(sc + S.part);
    const sdemc_inst* hinsts = reinterpret_cast<const sdemc_inst*>(hb + H.off_insts);
    B.uniform_seed = 1;
    for (int i = C.first + 1; i < C.first + C.count; ++i)
      if (hinsts[i].seed != hinsts[C.first].seed) { B.uniform_seed = 0; break; }
    if (B.uniform_seed && C.count > 0) B.rk = make_round_keys(hinsts[C.first].seed);
    const int64_t chunks = C.chunk_end - C.chunk_begin;
    if (chunks == 0) continue;
    cudaStream_t ks = n_side > 0 ? (cudaStream_t)side_streams[k % n_side] : s;
    rc = launch_class(C.dim, C.noise, C.mode, B, h_cfgs ? &h_cfgs[k] : nullptr, chunks, ks);
  }
  if (forked > 0) {
    const int err = rc;
    for (int j = 0; j < forked; ++j) {
      int jr = check_cuda(cudaEventRecord(ev->join[j], (cudaStream_t)side_streams[j]), "join record");
      if (jr == SDEMC_OK) jr = check_cuda(cudaStreamWaitEvent(s, ev->join[j], 0), "join wait");
      if (rc == SDEMC_OK) rc = jr;
    }
    if (err != SDEMC_OK) return err;
  }
  if (rc != SDEMC_OK) return rc;
  BatchReduceParams R;
  R.chunk_prefix = reinterpret_cast<const int64_t*>(db + H.off_chunk_prefix);
  R.group_prefix = reinterpret_cast<const int64_t*>(db + H.off_group_prefix);
  R.order = reinterpret_cast<const int32_t*>(db + H.off_order);
  R.n = H.n_inst;
  R.part = reinterpret_cast<const double*>(sc + S.part);
  R.groups = reinterpret_cast<double*>(sc + S.groups);
  R.status = reinterpret_cast<int32_t*>(sc + S.status);
  R.counters = reinterpret_cast<unsigned*>(sc + S.red_counters);
  R.out = d_out;
  if (H.total_groups > 0x7fffffff) return fail(SDEMC_EINVAL, "too many reduction groups");
  batch_reduce_kernel<<<(unsigned)H.total_groups, kGroup, 0, s>>>(R);
  return check_cuda(cudaGetLastError(), "batch_reduce_kernel launch");
}

// ------------------------------------------------------------- autotune ----
// Times sdemc_price_batch with CUDA events on `stream` (the plan blob must
// already be on the device): first every (block_threads, side streams)
// candidate, then, class by class, two paths per lane, kept when the whole
// batch gets more than 1% faster.  Best of `repeats` launches after one warm
// launch per setting.  Leaves d_out holding the last launch's results.
namespace sdemc {
static int time_batch(const void* h_blob, const void* d_blob, void* d_scratch, size_t scratch_bytes, double* d_out,
                      const sdemc_cfg* cfgs, void* const* side, int n_side, int repeats, cudaStream_t s,
                      cudaEvent_t e0, cudaEvent_t e1, float* ms) {
  int rc = sdemc_price_batch(h_blob, d_blob, d_scratch, scratch_bytes, d_out, cfgs, side, n_side, s);
  if (rc) return rc;
  float best = 3.4e38f;
  for (int r = 0; r < repeats; ++r) {
    if ((rc = check_cuda(cudaEventRecord(e0, s), "event record"))) return rc;
    if ((rc = sdemc_price_batch(h_blob, d_blob, d_scratch, scratch_bytes, d_out, cfgs, side, n_side, s))) return rc;
    if ((rc = check_cuda(cudaEventRecord(e1, s), "event record"))) return rc;
    if ((rc = check_cuda(cudaEventSynchronize(e1), "event sync"))) return rc;
    float t = 0.f;
    if ((rc = check_cuda(cudaEventElapsedTime(&t, e0, e1), "elapsed time"))) return rc;
    if (t < best) best = t;
  }
  *ms = best;
  return SDEMC_OK;
}
}  // namespace sdemc

extern "C" int sdemc_batch_autotune(const void* h_blob, const void* d_blob, void* d_scratch, size_t scratch_bytes,
                                    double* d_out, const int32_t* h_block_threads, const int32_t* h_side_counts,
                                    int n_cand, void* const* side_streams, int max_side, int repeats,
                                    sdemc_cfg* h_cfgs, int* h_n_side, float* h_ms, float* h_cand_ms,
                                    void* stream) {
  if (!h_blob || !h_block_threads || !h_side_counts || n_cand < 1 || !h_cfgs || !h_n_side || !h_ms || repeats < 1)
    return fail(SDEMC_EINVAL, "bad autotune arguments");
  const sdemc_batch_header& H = *static_cast<const sdemc_batch_header*>(h_blob);
  const int nc = H.n_class > 0 ? H.n_class : 1;
  for (int c = 0; c < n_cand; ++c) {
    if (h_side_counts[c] < 0 || h_side_counts[c] > max_side || (h_side_counts[c] > 0 && !side_streams))
      return fail(SDEMC_EINVAL, "candidate %d wants %d side streams (%d given)", c, h_side_counts[c], max_side);
    const int bt = h_block_threads[c];
    if (bt < 0 || bt > 256 || bt % 32) return fail(SDEMC_EINVAL, "candidate %d: block_threads %d", c, bt);
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = check_cuda(cudaEventCreate(&e0), "event create");
  if (!rc) rc = check_cuda(cudaEventCreate(&e1), "event create");
  float best = 3.4e38f;
  int best_c = 0;
  for (int c = 0; c < n_cand && !rc; ++c) {
    for (int k = 0; k < nc; ++k) h_cfgs[k] = sdemc_cfg{h_block_threads[c], 0, 1, 0, 0};
    float t = 0.f;
    rc = time_batch(h_blob, d_blob, d_scratch, scratch_bytes, d_out, h_cfgs, side_streams, h_side_counts[c],
                    repeats, s, e0, e1, &t);
    if (!rc && h_cand_ms) h_cand_ms[c] = t;
    if (!rc && t < best) { best = t; best_c = c; }
  }
  for (int k = 0; k < nc; ++k) h_cfgs[k] = sdemc_cfg{h_block_threads[best_c], 0, 1, 0, 0};
  for (int k = 0; k < H.n_class && !rc; ++k) {
    h_cfgs[k].interleave = 2;
    float t = 0.f;
    rc = time_batch(h_blob, d_blob, d_scratch, scratch_bytes, d_out, h_cfgs, side_streams, h_side_counts[best_c],
                    repeats, s, e0, e1, &t);
    if (!rc && t < 0.99f * best) best = t;
    else h_cfgs[k].interleave = 1;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc) return rc;
  *h_n_side = h_side_counts[best_c];
  *h_ms = best;
  return SDEMC_OK;
}
