// tl_walk.cuh -- the tile walk and the deterministic reduction tree shared by
// every kernel that reduces over the interior.
//
// Order (reproduced by the CPU restatement's device order):
//   1. tile t of (64*warps) columns x `rows` rows; block b walks t = b, b+G, ...
//   2. lane l of warp w adds its column pair i0 = 64*w + 2*l row by row
//      (cell i0 then i0+1) into a per-thread accumulator starting at 0.0;
//   3. xor butterfly over the warp (16, 8, 4, 2, 1);
//   4. warp sums added in warp order -> block partial;
//   5. the last block to finish (atomic ticket) adds the G partials: thread t
//      takes partials t, t+F, ... in order, then steps 3 and 4 again.
// The tree depends only on (nx, ny, warps, rows, G), never on timing.
#pragma once

#include "tl_internal.cuh"

namespace tl {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// a*x + y: rounded twice (exact: the reference's broadcast) or fused.
template <bool EXACT>
__device__ __forceinline__ double axpy(double a, double x, double y) {
  if (EXACT) return dadd(dmul(a, x), y);
  return fma(a, x, y);
}
// acc + x*y
template <bool EXACT>
__device__ __forceinline__ double acc_mul(double acc, double x, double y) {
  if (EXACT) return dadd(acc, dmul(x, y));
  return fma(x, y, acc);
}

__device__ __forceinline__ double2 ld2(const double *p) { return __ldg(reinterpret_cast<const double2 *>(p)); }
__device__ __forceinline__ void st2(double *p, double2 v) { *reinterpret_cast<double2 *>(p) = v; }

__device__ __forceinline__ double warp_butterfly(double v) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) v = dadd(v, __shfl_xor_sync(FULL, v, off));
  return v;
}

// Steps 3-5.  `fin(tot)` runs on thread 0 of the last block with the totals.
template <int N, class Op>
__device__ __forceinline__ void finish_reduction(double (&acc)[N], const Op &op) {
  __shared__ double ws[N][32];
  __shared__ int is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double *partials = op.F.partials;
  unsigned *counter = op.F.counter;
#pragma unroll
  for (int a = 0; a < N; ++a) {
    const double v = warp_butterfly(acc[a]);
    if (lane == 0) ws[a][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int a = 0; a < N; ++a) {
      double b = ws[a][0];
      for (int w = 1; w < nw; ++w) b = dadd(b, ws[a][w]);
      partials[(size_t)a * gridDim.x + blockIdx.x] = b;
    }
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
#pragma unroll
  for (int a = 0; a < N; ++a) {
    double v = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) v = dadd(v, __ldcg(partials + (size_t)a * gridDim.x + k));
    v = warp_butterfly(v);
    if (lane == 0) ws[a][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot[N];
#pragma unroll
    for (int a = 0; a < N; ++a) {
      tot[a] = ws[a][0];
      for (int w = 1; w < nw; ++w) tot[a] = dadd(tot[a], ws[a][w]);
    }
    *counter = 0u;
    op.fin(tot);
  }
}

// The walk.  Op provides: bool skip() (uniform early exit), void on_skip(),
// void tile(i0, j0, j1, acc), void fin(const double*) (N > 0), and Fields F.
template <int N, class Op>
__global__ void __launch_bounds__(256) k_walk(const Op op, const Walk wk, const int ny) {
  if (op.skip()) {
    op.on_skip();
    return;
  }
  constexpr int NA = N > 0 ? N : 1;
  double acc[NA];
#pragma unroll
  for (int a = 0; a < NA; ++a) acc[a] = 0.0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int TW = 64 * wk.warps;
  for (int t = blockIdx.x; t < wk.tiles; t += gridDim.x) {
    const int tx = t % wk.ntx, ty = t / wk.ntx;
    const int i0 = tx * TW + warp * 64 + 2 * lane;
    const int j0 = ty * wk.rows;
    const int j1 = min(j0 + wk.rows, ny);
    op.tile(i0, j0, j1, acc);
  }
  if constexpr (N > 0) finish_reduction<N>(acc, op);
}

template <int N, class Op>
inline void launch_walk(cudaStream_t st, const Op &op, const Walk &wk, int ny) {
  k_walk<N, Op><<<wk.blocks, 32 * wk.warps, 0, st>>>(op, wk, ny);
}

// Base for ops without an early exit.
struct NoSkip {
  __device__ bool skip() const { return false; }
  __device__ void on_skip() const {}
};

// The loop control shared by every iteration epilogue (runs on one thread).
// rule: 0 = CG test sqrt|error| < eps (CG.jl:24); 1 = |error| < eps plus the
// Cheby/PPCG switch rule (Cheby.jl:25-29, PPCG.jl:27-31); 2 = |error| < eps.
__device__ __forceinline__ void loop_control(DevScalars *sc, cudaGraphConditionalHandle h, int set_cond) {
  bool conv;
  if (sc->crit == TL_CRIT_RELATIVE)
    conv = sqrt(fabs(sc->error) / sc->bb) < sc->eps;
  else if (sc->switch_rule == 0)
    conv = sqrt(fabs(sc->error)) < sc->eps;
  else
    conv = fabs(sc->error) < sc->eps;
  bool sw = false;
  if (!conv && sc->switch_rule == 1) {
    const int tt = sc->iter + 1;  // next trip of the solver loop
    sw = sc->errorswitch ? (sc->error < sc->epslim) && (tt > CGEIGENITERS)
                         : (tt > sc->presteps) && (sc->error < ERROR_SWITCH_MAX);
  }
  sc->converged = conv;
  sc->switched = sw;
  const int done = conv || sw || sc->iter >= sc->maxiters;
  sc->done = done;
  if (set_cond) cudaGraphSetConditional(h, done ? 0u : 1u);
}

}  // namespace tl
