// k_store_kern.cuh — the kernels of K4 (materialised paths) and K3 (replay
// of recorded draws), shared by the translation units that instantiate them:
// k_store_diag.cu, k_store_indep_shared.cu and k_store_indep_pair.cu each
// compile the kernels of one noise layout (so the three compile in
// parallel), and k_store.cu holds the entry points.
#pragma once
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

struct StoreParams {
  sdemc_inst I;
  RoundKeys rk;
};

// AdaptedPathData stores through shared memory.  A path's rows are contiguous
// in every array, so a lane writing its own row at each step touches one
// 32-byte sector per lane and array for a few bytes; instead each lane parks
// kT steps of (paths, left, jumps, time, normals) in its warp's tile and the
// warp then writes lane after lane's kT-row segments with consecutive lanes on
// consecutive addresses.  Measured on the 2D rainbow (2^20 paths, 271 rows):
//   * the time follows the number of segments, so a tile holds up to 32 / D
//     steps (128 B of one path's state per segment; 64-B segments took 1.6x
//     as long, 32-B ones 3x), within 48 KB of static shared memory for the
//     CTA's two warps (one-warp CTAs with 256-B segments were slower);
//   * segments start on a row that is a multiple of kT (state row r in slot
//     r % kT, normals row k in slot k % kT), so when a path's row is a whole
//     number of lines every segment is whole lines and sectors: no partial
//     sector reaches DRAM (its read-modify-write had cost 25 % of the written
//     bytes in extra reads), 1.8x faster.
// The padding rows after the loop (the terminal state repeated to S, zero
// normals) go the same way.  Called in lock-step: k is the same in every lane
// of the warp.
constexpr int kStoreThreads = 64;
constexpr int kStoreLaneFloats = 48 * 1024 / 4 / kStoreThreads;  // 192

template <int D, int NW>
struct TiledStoreSink {
  static constexpr bool kWantsLeft = true;
  static constexpr int kRowW = 3 * D + 1;             // paths, left, jumps (D each), time
  static constexpr int kNw = D * NW;                  // normals per step
  static constexpr int kW = kRowW + kNw;
  static constexpr int kTWant = (32 / D) > 2 ? 32 / D : 2;
  static constexpr int odd_stride(int kt) { return kt * kW + ((kt * kW) % 2 == 0 ? 1 : 2); }
  // rows per tile; the lane stride is odd, so a lane's writes and the flush
  // reads spread over the banks
  static constexpr int kT = odd_stride(kTWant) <= kStoreLaneFloats ? kTWant : (kTWant / 2 > 2 ? kTWant / 2 : 2);
  static constexpr int kLaneStride = odd_stride(kT);
  static_assert(kLaneStride <= kStoreLaneFloats, "tile exceeds the static shared memory");
  static constexpr int kTileFloats = 32 * kLaneStride;
  float *paths, *left, *time, *jumps, *normals;
  float* tile;       // this warp's 32 lanes x kLaneStride floats
  int64_t p0;        // path of lane 0
  int64_t n;         // num_paths
  int S;

  SDEMC_DI float& at(int kk, int lane, int f) const { return tile[lane * kLaneStride + kk * kW + f]; }

  // Row 0 of the state arrays (x0, x0, 0, t = 0) goes to tile slot 0: state
  // row r lives in slot r % kT and normals row k in slot k % kT, so every
  // flush writes rows that start on a multiple of kT.
  template <int Dd> SDEMC_DI void init(const float* x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      at(0, lane, i) = x[i];
      at(0, lane, D + i) = x[i];
      at(0, lane, 2 * D + i) = 0.f;
    }
    at(0, lane, 3 * D) = 0.f;
  }

  // One array's segments: every lane's rows [r0, r0 + cnt) of width W, from
  // tile column f0 on.  CNT > 0: a full tile (cnt = CNT, so the index
  // arithmetic divides by constants); CNT = 0: a partial tile of cnt rows.
  template <int W, int CNT>
  SDEMC_DI void put(float* base, int rows, int f0, int r0, int cnt) const {
    if (!base) return;
    const int lane = threadIdx.x & 31;
    constexpr int SEG = CNT * W;
    constexpr int SEGD = SEG > 0 ? SEG : 1;  // the divisor when the branch below is live
    if (CNT > 0 && SEG <= 32 && (32 % SEGD) == 0) {
      // a full tile whose segments tile the warp: every lane keeps one
      // (row, column) of the segment and walks the paths
      constexpr int PPI = 32 / SEGD;  // paths per store instruction
      const int q = lane % SEGD, kk = q / W, f = q - kk * W;
      const int jl = lane / SEGD;
      const float* src = tile + jl * kLaneStride + kk * kW + f0 + f;  // path jl; + it * PPI paths
      float* dst = base + ((size_t)(p0 + jl) * rows + r0 + kk) * W + f;
      const size_t step = (size_t)PPI * rows * W;
      if (n - p0 >= 32) {  // warp-uniform: every path of the warp is in range
#pragma unroll
        for (int it = 0; it < SEG; ++it) {
          *dst = src[it * PPI * kLaneStride];
          dst += step;
        }
      } else {
        const int live = (int)(n - p0);  // paths of the warp in range (< 32)
#pragma unroll
        for (int it = 0; it < SEG; ++it) {
          if (it * PPI + jl < live) *dst = src[it * PPI * kLaneStride];
          dst += step;
        }
      }
      return;
    }
    const int seg = (CNT > 0 ? CNT : cnt) * W;
#pragma unroll 4
    for (int e = lane; e < 32 * seg; e += 32) {
      const int j = e / seg, r = e - j * seg, kk = r / W, f = r - kk * W;
      const int64_t p = p0 + j;
      if (p < n) base[((size_t)p * rows + r0 + kk) * W + f] = at(kk, j, f0 + f);
    }
  }

  // State rows [r0, r0 + cnt) (r0 a multiple of kT) from slots 0 .. cnt-1.
  template <int CNT>
  SDEMC_DI void flush_state(int r0, int cnt) const {
    __syncwarp();
    put<D, CNT>(paths, S + 1, 0, r0, cnt);
    put<D, CNT>(left, S + 1, D, r0, cnt);
    put<D, CNT>(jumps, S + 1, 2 * D, r0, cnt);
    put<1, CNT>(time, S + 1, 3 * D, r0, cnt);
    __syncwarp();
  }
  // Normals rows [k0, k0 + cnt) (k0 a multiple of kT).
  template <int CNT>
  SDEMC_DI void flush_normals(int k0, int cnt) const {
    __syncwarp();
    put<kNw, CNT>(normals, S, kRowW, k0, cnt);
    __syncwarp();
  }

  SDEMC_DI void put_state(int s, int lane, const float* x, const float* xl, float J, int sel, int jump_one,
                          float t) const {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      at(s, lane, i) = x[i];
      at(s, lane, D + i) = xl[i];
      at(s, lane, 2 * D + i) = (jump_one && i != sel) ? 0.f : J;
    }
    at(s, lane, 3 * D) = t;
  }

  // Step k writes state row k + 1 and normals row k; a slot group that is
  // full is written out.
  template <int Dd, int NWd>
  SDEMC_DI void step(int k, const float* xl, const float* x, float t, float J, int sel,
                     const float* dW, const float* dW2, const float*, int jump_one, const float*, float) {
    if (k >= S) return;
    const int lane = threadIdx.x & 31, sn = k % kT, ss = (k + 1) % kT;
    put_state(ss, lane, x, xl, J, sel, jump_one, t);
#pragma unroll
    for (int i = 0; i < D; ++i) {
      if (NW == 1) {
        at(sn, lane, kRowW + i) = dW[i];
      } else {
        at(sn, lane, kRowW + 2 * i) = dW[i];
        at(sn, lane, kRowW + 2 * i + 1) = dW2[i];
      }
    }
    if (ss == kT - 1) flush_state<kT>(k + 2 - kT, kT);
    if (sn == kT - 1) flush_normals<kT>(k + 1 - kT, kT);
  }

  // Steps kend .. S-1 are padding: the terminal state (x, x, 0, t) in state
  // rows kend + 1 .. S and zero normals in rows kend .. S-1; then the open
  // slot groups are written out.
  template <int Dd, int NWd>
  SDEMC_DI void finish(int kend, const float* x, float t) {
    const int lane = threadIdx.x & 31;
    if (kend > S) kend = S;
    for (int k = kend; k < S; ++k) {
      const int sn = k % kT, ss = (k + 1) % kT;
      put_state(ss, lane, x, x, 0.f, 0, 0, t);
#pragma unroll
      for (int i = 0; i < kNw; ++i) at(sn, lane, kRowW + i) = 0.f;
      if (ss == kT - 1) flush_state<kT>(k + 2 - kT, kT);
      if (sn == kT - 1) flush_normals<kT>(k + 1 - kT, kT);
    }
    // rows 0 .. S of the state and 0 .. S-1 of the normals are in the tile or
    // written; the last groups are partial unless they end on a multiple of kT
    if ((S + 1) % kT != 0) flush_state<0>(S + 1 - (S + 1) % kT, (S + 1) % kT);
    if (S % kT != 0) flush_normals<0>(S - S % kT, S % kT);
  }

};

// EXPORT: the raw draws and the jump stream are exported for the oracle
// (per-lane row stores); otherwise the tiled stores only, compiled apart so the
// export code adds no registers to the layout kernel.
template <int D, int NOISE, int MODE, bool EXPORT>
__global__ void __launch_bounds__(kStoreThreads)
materialise_kernel(const __grid_constant__ StoreParams P, int S, float* paths, float* left,
                   float* time, float* jumps, float* normals, float* payoffs, int32_t* steps,
                   float* zout, int zdim, float* jt, float* jm, int32_t* jsel, int jcap,
                   int32_t* status, int max_iters) {
  using L = Layout<D, NOISE>;
  using Tiled = TiledStoreSink<D, L::NW>;
  __shared__ float tiles[kStoreThreads / 32][Tiled::kTileFloats];
  const sdemc_inst& I = P.I;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < I.num_paths;
  NativeDraws<D, NOISE> dr;
  dr.init(I, (uint64_t)p, ConstKeys{&P.rk});
  bool ovf = false;
  float x[D];
  const int it = max_iters < S ? max_iters : S;
  int own;
  if constexpr (!EXPORT) {
    Tiled sk;
    sk.paths = paths; sk.left = left; sk.time = time; sk.jumps = jumps; sk.normals = normals;
    sk.tile = tiles[threadIdx.x >> 5];
    sk.p0 = p - (threadIdx.x & 31);
    sk.n = I.num_paths;
    sk.S = S;
    own = simulate<D, NOISE, MODE>(I, dr, sk, x, it, ovf);
  } else {
    // with the raw draws exported (the oracle's step-by-step check): per-lane rows
    StoreSink sk{};
    sk.S = S;
    sk.zdim = zdim;
    if (valid) {
      const size_t row = (size_t)p * (S + 1);
      sk.paths = paths ? paths + row * D : nullptr;
      sk.left = left ? left + row * D : nullptr;
      sk.time = time ? time + row : nullptr;
      sk.jumps = jumps ? jumps + row * D : nullptr;
      sk.normals = normals ? normals + (size_t)p * S * D * L::NW : nullptr;
      sk.z = zout ? zout + (size_t)p * S * zdim : nullptr;
    }
    own = simulate<D, NOISE, MODE>(I, dr, sk, x, it, ovf);
  }
  if (!valid) return;
  if (payoffs) payoffs[p] = __fmul_rn(payoff<D>(I, x), I.discount);
  if (steps) steps[p] = own;
  if (ovf) atomicOr(status, SDEMC_EOVERFLOW);
  // Export the jump stream (times, marks, picks) for the oracle: blocks 0, 1,
  // 2, ... of the path's jump stream, times accumulated as the loop does.
  if (EXPORT && jcap > 0 && (jt || jm || jsel)) {
    float nj = inf_f();
    for (int j = 0; j < jcap; ++j) {
      JumpDraw d{0.f, 0.f, 0};
      if (I.rate > 0.f) {
        d = jump_from_block<D>(I, dr.ps.block(kTagJumps, (uint32_t)j));
        nj = j == 0 ? d.gap : __fadd_rn(nj, d.gap);
      }
      if (jt) jt[(size_t)p * jcap + j] = nj;
      if (jm) jm[(size_t)p * jcap + j] = d.mark;
      if (jsel) jsel[(size_t)p * jcap + j] = d.sel;
    }
  }
}

template <int D, int NOISE>
__global__ void __launch_bounds__(128)
replay_kernel(const __grid_constant__ sdemc_inst I, int bs, int S, int MJ, const float* jt,
              const float* dw, const float* marks, const int32_t* asset, float* paths,
              float* left, float* time, float* jumps, float* payoffs, int32_t* steps,
              int32_t* status) {
  using L = Layout<D, NOISE>;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < bs;
  StoreSink sk{};
  sk.S = S;
  sk.zdim = 0;
  ReplayDraws<D, NOISE> dr{};
  dr.S = 0;
  dr.MJ = 0;
  if (valid) {
    const size_t row = (size_t)p * (S + 1);
    sk.paths = paths + row * D;
    sk.left = left ? left + row * D : nullptr;
    sk.time = time ? time + row : nullptr;
    sk.jumps = jumps ? jumps + row * D : nullptr;
    dr.dw = dw + (size_t)p * S * D * L::NW;
    dr.marks = marks ? marks + (size_t)p * S : nullptr;
    dr.asset = asset ? asset + (size_t)p * S : nullptr;
    dr.jt = jt ? jt + (size_t)p * MJ : nullptr;
    dr.S = S;
    dr.MJ = jt ? MJ : 0;
  }
  dr.overflow = false;
  bool ovf = false;
  float x[D];
  const int own = simulate<D, NOISE, kModeExact>(I, dr, sk, x, S, ovf);
  if (!valid) return;
  if (payoffs) payoffs[p] = __fmul_rn(payoff<D>(I, x), I.discount);
  if (steps) steps[p] = own;
  if (ovf || dr.overflow) atomicOr(status, SDEMC_EOVERFLOW);
}

// K4 launch of every dimension and loop variant of one noise layout (zdim is
// checked by the caller); instantiated once per layout.
template <int NOISE>
int launch_materialise_noise(const StoreParams& P, bool nominal, unsigned blocks, int steps_cap, float* d_paths,
                             float* d_left, float* d_time, float* d_jumps, float* d_normals, float* d_payoffs,
                             int32_t* d_steps, float* d_z, float* d_jt, float* d_jm, int32_t* d_jsel, int jcap,
                             int32_t* d_status, int mi, cudaStream_t s) {
  const bool exporting = d_z != nullptr || (jcap > 0 && (d_jt || d_jm || d_jsel));
#define SDEMC_MAT_CASE(D_, N_)                                                                      \
  {                                                                                                 \
    constexpr int ZD = Layout<D_, N_>::ZD;                                                          \
    auto kern = nominal ? (exporting ? materialise_kernel<D_, N_, kModeNominal, true>                     \
                               : materialise_kernel<D_, N_, kModeNominal, false>)                    \
                        : (exporting ? materialise_kernel<D_, N_, 0, true> : materialise_kernel<D_, N_, 0, false>); \
    kern<<<blocks, kStoreThreads, 0, s>>>(P, steps_cap, d_paths, d_left, d_time, d_jumps, d_normals, d_payoffs, \
                                d_steps, d_z, ZD, d_jt, d_jm, d_jsel, jcap, d_status, mi);           \
  }
  SDEMC_DISPATCH_DIM(NOISE, P.I.dim, SDEMC_MAT_CASE)
#undef SDEMC_MAT_CASE
  return check_cuda(cudaGetLastError(), "materialise_kernel launch");
}

// K3 launch of every dimension of one noise layout.
template <int NOISE>
int launch_replay_noise(const sdemc_inst& I, unsigned blocks, int bs, int steps_cap, int max_jumps,
                        const float* d_jump_times, const float* d_dw, const float* d_marks, const int32_t* d_asset,
                        float* d_paths, float* d_left, float* d_time, float* d_jumps, float* d_payoffs,
                        int32_t* d_steps, int32_t* d_status, cudaStream_t s) {
#define SDEMC_REPLAY_CASE(D_, N_)                                                                          \
  replay_kernel<D_, N_><<<blocks, 128, 0, s>>>(I, bs, steps_cap, max_jumps, d_jump_times, d_dw, d_marks, \
                                               d_asset, d_paths, d_left, d_time, d_jumps, d_payoffs,     \
                                               d_steps, d_status);
  SDEMC_DISPATCH_DIM(NOISE, I.dim, SDEMC_REPLAY_CASE)
#undef SDEMC_REPLAY_CASE
  return check_cuda(cudaGetLastError(), "replay_kernel launch");
}

#define SDEMC_MATERIALISE_NOISE_SIG(N_)                                                                      \
  int launch_materialise_noise<N_>(const StoreParams&, bool, unsigned, int, float*, float*, float*, float*, \
                                   float*, float*, int32_t*, float*, float*, float*, int32_t*, int, int32_t*, \
                                   int, cudaStream_t)
#define SDEMC_REPLAY_NOISE_SIG(N_)                                                                            \
  int launch_replay_noise<N_>(const sdemc_inst&, unsigned, int, int, int, const float*, const float*,         \
                              const float*, const int32_t*, float*, float*, float*, float*, float*, int32_t*, \
                              int32_t*, cudaStream_t)
extern template SDEMC_MATERIALISE_NOISE_SIG(SDEMC_NOISE_DIAG);
extern template SDEMC_MATERIALISE_NOISE_SIG(SDEMC_NOISE_INDEP_SHARED);
extern template SDEMC_MATERIALISE_NOISE_SIG(SDEMC_NOISE_INDEP_PAIR);
extern template SDEMC_REPLAY_NOISE_SIG(SDEMC_NOISE_DIAG);
extern template SDEMC_REPLAY_NOISE_SIG(SDEMC_NOISE_INDEP_SHARED);
extern template SDEMC_REPLAY_NOISE_SIG(SDEMC_NOISE_INDEP_PAIR);

}  // namespace sdemc
