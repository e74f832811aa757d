// tl_batch.cu -- many independent decks of uneven sizes solved by CG in one
// graph launch.
//
// Every deck keeps its own context (fields, scalars, reduction scratch).  The
// batch owns a device table of the decks and a block map: the persistent
// blocks of each batched kernel are split over the unconverged decks in
// proportion to their cells (at least one each).  A batched kernel's block
// looks up its deck, walks that deck's tiles with the deck's share of blocks
// and reduces into the deck's scratch; the last block of a deck runs the
// deck's epilogue (alpha, or beta and the convergence test).  A converged
// deck's blocks return at once (the per-deck convergence mask), and at the end
// of every two-iteration loop body the map is rebuilt over the decks still
// running, which also sets the while-node's condition.
//
// With FP32 refinement the body runs two FP32 inner iterations for the decks
// in their inner loop, then the FP64 refinement step (u += x, halo of u, true
// residual, test) for the decks whose inner loop just ended; the test either
// finishes the deck or restarts its inner loop from the true residual, all on
// the device.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "tl_cg_ops.cuh"
#include "tl_ir_ops.cuh"
#include "tl_solvers.h"

namespace tl {
namespace {

constexpr int BATCH_MAX = 1024;  // decks per batch
constexpr int BATCH_WARPS = 8;
constexpr int BATCH_ROWS = 8;
constexpr int BATCH_ROWS32 = 32;  // rows of an FP32 warp tile: longer walks hide the row prefetch's latency

// Work is handed out per warp: a warp tile is one warp's column strip (64
// columns for the FP64 kernels, 128 for the FP32 ones) over BATCH_ROWS rows,
// and the warps of a deck's blocks take its warp tiles in turn.  Narrow decks
// then keep every warp busy.
struct DeckDesc {
  Fields F;
  Geom g;
  int ntx, tiles;           // FP64 warp tiles: per row band, and in all
  long long cells;
  // FP32 refinement buffers (filled on the first batched FP32 solve)
  G32 g32;
  IrPtrs q;
  float *p32, *pb32;
  int ntx32, tiles32;       // FP32 warp tiles
};

struct BatchMap {
  int n;
  int active;
  int total_w, total_u;     // blocks of the W and UR launches
  int first_w[BATCH_MAX + 1], nblk_w[BATCH_MAX];
  int first_u[BATCH_MAX + 1], nblk_u[BATCH_MAX];
  int first_r[BATCH_MAX + 1], nblk_r[BATCH_MAX];  // FP32 refinement: all blocks over the refining decks
};

__device__ __forceinline__ int find_deck(const int *first, const int *nblk, int n, int b) {
  int lo = 0, hi = n - 1, d = -1;
  while (lo <= hi) {  // last deck whose first block is <= b
    const int mid = (lo + hi) >> 1;
    if (first[mid] <= b) {
      d = mid;
      lo = mid + 1;
    } else {
      hi = mid - 1;
    }
  }
  if (d >= 0 && b < first[d] + nblk[d]) return d;
  return -1;
}

// The deterministic tree of tl_walk.cuh, over a deck's own blocks.
template <int N, class Op>
__device__ __forceinline__ void finish_deck(double (&acc)[N], const Op &op, int nblocks, int lb) {
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
      partials[(size_t)a * nblocks + lb] = b;
    }
    __threadfence();
    is_last = (atomicAdd(counter, 1u) == (unsigned)nblocks - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
#pragma unroll
  for (int a = 0; a < N; ++a) {
    double v = 0.0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) v = dadd(v, __ldcg(partials + (size_t)a * nblocks + k));
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

template <class Op>
__device__ __forceinline__ void walk_deck(const DeckDesc &D, const Op &op, int lb, int nblocks, double (&acc)[1]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int t = lb * nw + warp; t < D.tiles; t += nblocks * nw) {
    const int tx = t % D.ntx, ty = t / D.ntx;
    const int i0 = tx * 64 + 2 * lane;
    const int j0 = ty * BATCH_ROWS;
    const int j1 = min(j0 + BATCH_ROWS, D.g.ny);
    op.tile(i0, j0, j1, acc);
  }
}

// W step of every unconverged deck: p' = beta p + r, w = A p', p'.w.
__global__ void __launch_bounds__(256) k_batch_w(const DeckDesc *decks, const BatchMap *map, int parity) {
  const int d = find_deck(map->first_w, map->nblk_w, map->n, blockIdx.x);
  if (d < 0) return;
  const DeckDesc &D = decks[d];
  if (D.F.sc->done) return;  // the deck's convergence mask: uniform over its blocks
  OpTlW<false> op;
  op.F = D.F;
  op.g = D.g;
  op.psrc = parity ? D.F.pb : D.F.p;
  op.pdst = parity ? D.F.p : D.F.pb;
  op.guard = 0;
  op.store_coef = 1;
  double acc[1] = {0.0};
  const int lb = blockIdx.x - map->first_w[d], nb = map->nblk_w[d];
  walk_deck(D, op, lb, nb, acc);
  finish_deck<1>(acc, op, nb, lb);
}

// UR step of every unconverged deck: u += alpha p', r -= alpha w, r.r, then
// the deck's beta and convergence test.
__global__ void __launch_bounds__(256) k_batch_ur(const DeckDesc *decks, const BatchMap *map, int parity) {
  const int d = find_deck(map->first_u, map->nblk_u, map->n, blockIdx.x);
  if (d < 0) return;
  const DeckDesc &D = decks[d];
  if (D.F.sc->done) return;
  OpTlUR<false> op;
  op.F = D.F;
  op.g = D.g;
  op.p = parity ? D.F.p : D.F.pb;
  op.guard = 0;
  op.cond = 0;
  op.set_cond = 0;
  double acc[1] = {0.0};
  const int lb = blockIdx.x - map->first_u[d], nb = map->nblk_u[d];
  walk_deck(D, op, lb, nb, acc);
  finish_deck<1>(acc, op, nb, lb);
}

// ---- FP32 refinement --------------------------------------------------------

// Walk with four cells per lane over the deck's FP32 warp tiles.
template <class Op>
__device__ __forceinline__ void walk_deck32(const DeckDesc &D, const Op &op, int lb, int nblocks, double (&acc)[1]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int t = lb * nw + warp; t < D.tiles32; t += nblocks * nw) {
    const int tx = t % D.ntx32, ty = t / D.ntx32;
    const int i0 = tx * 128 + 4 * lane;
    const int j0 = ty * BATCH_ROWS32;
    const int j1 = min(j0 + BATCH_ROWS32, D.g.ny);
    op.tile(i0, j0, j1, acc);
  }
}

// FP32 direction step of every deck in its inner loop: p' = beta p + r,
// p'.A p', p' stored.
__global__ void __launch_bounds__(256) k_batch_ir_w(const DeckDesc *decks, const BatchMap *map, int parity) {
  const int d = find_deck(map->first_w, map->nblk_w, map->n, blockIdx.x);
  if (d < 0) return;
  const DeckDesc &D = decks[d];
  if (D.F.sc->done) return;
  OpIrDir<2> op;
  op.F = D.F;
  op.g = D.g32;
  op.q = D.q;
  op.psrc = parity ? D.pb32 : D.p32;
  op.pdst = parity ? D.p32 : D.pb32;
  op.guard = 0;
  double acc[1] = {0.0};
  const int lb = blockIdx.x - map->first_w[d], nb = map->nblk_w[d];
  walk_deck32(D, op, lb, nb, acc);
  finish_deck<1>(acc, op, nb, lb);
}

// The FP32 update step's epilogue, plus where the search direction ended:
// after the even step it is in the second buffer.
struct OpIrUpdateBatch : OpIrUpdate<1> {
  int parity;
  __device__ void fin(const double *tot) const {
    OpIrUpdate<1>::fin(tot);
    if (F.sc->done) F.sc->pbuf = parity == 0 ? 1 : 0;
  }
};

// FP32 update step: A p' recomputed, x += alpha p', r -= alpha A p', r.r,
// beta, and the refinement test.
__global__ void __launch_bounds__(256) k_batch_ir_ur(const DeckDesc *decks, const BatchMap *map, int parity) {
  const int d = find_deck(map->first_u, map->nblk_u, map->n, blockIdx.x);
  if (d < 0) return;
  const DeckDesc &D = decks[d];
  if (D.F.sc->done) return;
  OpIrUpdateBatch op;
  op.F = D.F;
  op.g = D.g32;
  op.s = parity ? D.p32 : D.pb32;
  op.iw = D.q.iw;
  op.a = D.q.x;
  op.b = D.q.r;
  op.out = nullptr;
  op.pp = 0;
  op.guard = 0;
  op.cond = 0;
  op.set_cond = 0;
  op.parity = parity;
  double acc[1] = {0.0};
  const int lb = blockIdx.x - map->first_u[d], nb = map->nblk_u[d];
  walk_deck32(D, op, lb, nb, acc);
  finish_deck<1>(acc, op, nb, lb);
}

// A deck whose inner loop has ended and whose solve is not over.
__device__ __forceinline__ bool refining(const DeckDesc &D) { return D.F.sc->done && !D.F.sc->finished; }

// Refinement, FP64: u += x, x = 0; the current search direction moves to the
// first buffer.
__global__ void k_batch_ir_fold(const DeckDesc *decks, const BatchMap *map) {
  const int d = find_deck(map->first_r, map->nblk_r, map->n, blockIdx.x);
  if (d < 0) return;
  const DeckDesc &D = decks[d];
  if (!refining(D)) return;
  const int lb = blockIdx.x - map->first_r[d], nb = map->nblk_r[d];
  const bool move = D.F.sc->pbuf != 0;
  const long long n = (long long)D.g.nx * D.g.ny;
  for (long long k = (long long)lb * blockDim.x + threadIdx.x; k < n; k += (long long)nb * blockDim.x) {
    const int i = (int)(k % D.g.nx), j = (int)(k / D.g.nx);
    const size_t c = D.g.at(i, j), c32 = D.g32.at(i, j);
    D.F.u[c] = D.F.u[c] + (double)D.q.x[c32];
    D.q.x[c32] = 0.f;
    if (move) D.p32[c32] = D.pb32[c32];
  }
}

// Refinement: the reflective halo of u, depth 1, faces only (corners untouched).
__global__ void k_batch_ir_halo(const DeckDesc *decks, const BatchMap *map) {
  const int d = find_deck(map->first_r, map->nblk_r, map->n, blockIdx.x);
  if (d < 0) return;
  const DeckDesc &D = decks[d];
  if (!refining(D)) return;
  const int lb = blockIdx.x - map->first_r[d], nb = map->nblk_r[d];
  const int nx = D.g.nx, ny = D.g.ny;
  double *u = D.F.u;
  for (int k = lb * blockDim.x + threadIdx.x; k < 2 * (nx + ny); k += nb * blockDim.x) {
    if (k < ny) u[D.g.at(-1, k)] = u[D.g.at(0, k)];
    else if (k < 2 * ny) u[D.g.at(nx, k - ny)] = u[D.g.at(nx - 1, k - ny)];
    else if (k < 2 * ny + nx) u[D.g.at(k - 2 * ny, -1)] = u[D.g.at(k - 2 * ny, 0)];
    else u[D.g.at(k - 2 * ny - nx, ny)] = u[D.g.at(k - 2 * ny - nx, ny - 1)];
  }
}

// Refinement: the true residual r = u0 - A u (FP64), r32 = (float) r, and the
// test: the deck finishes (converged, or out of iterations) or its inner loop
// restarts from the true residual with the search direction kept.
struct OpIrResidBatch : OpIrResid {
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    const double rr = tot[0];
    const double rel = sc->bb > 0 ? sqrt(rr / sc->bb) : sqrt(rr);
    sc->red[0] = rr;
    sc->red[1] = rel;
    sc->refinements += 1;
    if (rel < sc->eps || sc->iter >= sc->maxiters) {
      sc->finished = 1;
      sc->converged = rel < sc->eps;
    } else {
      sc->rro = rr;
      sc->rr_ref = rr;
      sc->done = 0;
      sc->switched = 0;
      sc->pbuf = 0;
    }
  }
};

__global__ void __launch_bounds__(256) k_batch_ir_resid(const DeckDesc *decks, const BatchMap *map) {
  const int d = find_deck(map->first_r, map->nblk_r, map->n, blockIdx.x);
  if (d < 0) return;
  const DeckDesc &D = decks[d];
  if (!refining(D)) return;
  OpIrResidBatch op;
  op.F = D.F;
  op.g = D.g;
  op.g32 = D.g32;
  op.r32 = D.q.r;
  double acc[1] = {0.0};
  const int lb = blockIdx.x - map->first_r[d], nb = map->nblk_r[d];
  walk_deck(D, op, lb, nb, acc);
  finish_deck<1>(acc, op, nb, lb);
}

// Start of a deck's FP32-refined solve (after tea_leaf_init, copyu! and the
// FP32 copies): the first refinement reference and the initial test.
__global__ void k_batch_ir_start(DevScalars *sc, double delta2) {
  const double rr = sc->rro;
  const double rel = sc->bb > 0 ? sqrt(rr / sc->bb) : sqrt(rr);
  sc->rr_ref = rr;
  sc->delta2 = delta2;
  sc->switched = 0;
  sc->pbuf = 0;
  sc->refinements = 0;
  sc->red[0] = rr;
  sc->red[1] = rel;
  const int fin = rel < sc->eps || sc->maxiters < 1;
  sc->finished = fin;
  sc->done = fin;
  sc->converged = rel < sc->eps;
}

// Shares `total` blocks over the unconverged decks in proportion to their
// cells: one each, the rest in proportion (rounded down), at most as many
// blocks as the deck's warp tiles can fill.
__device__ void share(const DeckDesc *decks, BatchMap *map, const int *act, int total, int *first, int *nblk) {
  __shared__ long long cells_sum;
  __shared__ int spare;
  const int n = map->n;
  if (threadIdx.x == 0) {
    long long s = 0;
    int na = 0;
    for (int d = 0; d < n; ++d)
      if (act[d]) {
        s += decks[d].cells;
        ++na;
      }
    cells_sum = s;
    spare = total - na;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < n; d += blockDim.x) {
    int b = 0;
    if (act[d]) {
      const double want = cells_sum > 0 ? (double)spare * (double)decks[d].cells / (double)cells_sum : 0.0;
      b = 1 + (int)want;
      const int cap = (decks[d].tiles + BATCH_WARPS - 1) / BATCH_WARPS;  // every block has a warp tile
      if (b > cap) b = cap;
    }
    nblk[d] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int f = 0;
    for (int d = 0; d < n; ++d) {
      first[d] = f;
      f += nblk[d];
    }
    first[n] = f;
  }
  __syncthreads();
}

// Shares the blocks of the refinement kernels over the decks whose inner loop
// has just ended, so that a refinement runs on the whole GPU and not on one
// deck's share of it.
__global__ void k_batch_refine_map(const DeckDesc *decks, BatchMap *map) {
  __shared__ int act[BATCH_MAX];
  for (int d = threadIdx.x; d < map->n; d += blockDim.x) act[d] = refining(decks[d]) ? 1 : 0;
  __syncthreads();
  share(decks, map, act, map->total_w, map->first_r, map->nblk_r);
}

// Rebuilds the block map over the decks still running and sets the loop
// condition (any deck left).  A deck runs until `done` (FP64) or `finished`
// (FP32 refinement, where `done` only ends an inner loop).
__global__ void k_batch_map(const DeckDesc *decks, BatchMap *map, cudaGraphConditionalHandle cond, int set_cond,
                            int ir) {
  __shared__ int act[BATCH_MAX];
  __shared__ int nact;
  const int n = map->n;
  if (threadIdx.x == 0) nact = 0;
  __syncthreads();
  for (int d = threadIdx.x; d < n; d += blockDim.x) {
    act[d] = (ir ? decks[d].F.sc->finished : decks[d].F.sc->done) ? 0 : 1;
    if (act[d]) atomicAdd(&nact, 1);
  }
  __syncthreads();
  share(decks, map, act, map->total_w, map->first_w, map->nblk_w);
  share(decks, map, act, map->total_u, map->first_u, map->nblk_u);
  if (threadIdx.x == 0) {
    map->active = nact;
    if (set_cond) cudaGraphSetConditional(cond, nact > 0 ? 1u : 0u);
  }
}

}  // namespace
}  // namespace tl

using namespace tl;

struct tl_batch {
  std::vector<tl_ctx *> ctx;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  DeckDesc *d_decks = nullptr;
  BatchMap *d_map = nullptr;
  BatchMap *h_map = nullptr;
  int total_w = 0, total_u = 0;
  cudaGraphExec_t graph = nullptr;     // FP64 CG loop
  cudaGraphExec_t graph_ir = nullptr;  // FP32-refined CG loop
  int ir_ready = 0;                    // the deck table holds the FP32 buffers
  std::vector<DeckDesc> h_decks;
  double last_ms = 0.0;
  char msg[512] = {};
};

namespace {

int bfail(tl_batch *b, cudaError_t e, const char *what) {
  snprintf(b->msg, sizeof b->msg, "CUDA error in %s: %s", what, cudaGetErrorString(e));
  return TL_ERR_CUDA;
}
#define BCK(x)                                  \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return bfail(b, e_, #x); \
  } while (0)

// One trip of the batched loop: two CG iterations of every running deck,
// (FP32 refinement) the refinement of the decks whose inner loop ended, and
// the new block map with the loop condition.
void launch_body(tl_batch *b, int ir, cudaGraphConditionalHandle h, int set_cond) {
  for (int parity = 0; parity < 2; ++parity) {
    if (ir) {
      k_batch_ir_w<<<b->total_w, 256, 0, b->stream>>>(b->d_decks, b->d_map, parity);
      k_batch_ir_ur<<<b->total_u, 256, 0, b->stream>>>(b->d_decks, b->d_map, parity);
    } else {
      k_batch_w<<<b->total_w, 256, 0, b->stream>>>(b->d_decks, b->d_map, parity);
      k_batch_ur<<<b->total_u, 256, 0, b->stream>>>(b->d_decks, b->d_map, parity);
    }
  }
  if (ir) {
    k_batch_refine_map<<<1, 256, 0, b->stream>>>(b->d_decks, b->d_map);
    k_batch_ir_fold<<<b->total_w, 256, 0, b->stream>>>(b->d_decks, b->d_map);
    k_batch_ir_halo<<<b->total_w, 256, 0, b->stream>>>(b->d_decks, b->d_map);
    k_batch_ir_resid<<<b->total_w, 256, 0, b->stream>>>(b->d_decks, b->d_map);
  }
  k_batch_map<<<1, 256, 0, b->stream>>>(b->d_decks, b->d_map, h, set_cond, ir);
}

// The loop: the while-node graph, or (TEALEAF_GB300_LOOP=host, for
// profilers, which cannot see kernels inside graphs that hold conditional
// nodes) the same trips launched from the host in batches of eight until the
// map reports no running deck.  Trips after the last deck finished find no
// blocks assigned and return at once.
int run_loop(tl_batch *b, int ir) {
  const char *loop = getenv("TEALEAF_GB300_LOOP");
  if (!(loop && !strcmp(loop, "host"))) {
    BCK(cudaGraphLaunch(ir ? b->graph_ir : b->graph, b->stream));
    return TL_OK;
  }
  for (;;) {
    for (int t = 0; t < 8; ++t) launch_body(b, ir, 0, 0);
    BCK(cudaGetLastError());
    int active = 0;
    BCK(cudaMemcpyAsync(&active, &b->d_map->active, sizeof active, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    if (active == 0) return TL_OK;
  }
}

int build_graph(tl_batch *b, int ir) {
  cudaGraph_t graph = nullptr;
  BCK(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle h;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return bfail(b, e, "cudaGraphConditionalHandleCreate");
  }
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return bfail(b, e, "cudaGraphAddNode(while)");
  }
  cudaGraph_t body = np.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(b->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return bfail(b, e, "cudaStreamBeginCaptureToGraph");
  }
  launch_body(b, ir, h, 1);
  cudaError_t le = cudaGetLastError();
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(b->stream, &captured);
  if (e != cudaSuccess || le != cudaSuccess) {
    cudaGraphDestroy(graph);
    return bfail(b, e != cudaSuccess ? e : le, "capture of the batch loop");
  }
  e = cudaGraphInstantiate(ir ? &b->graph_ir : &b->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return bfail(b, e, "cudaGraphInstantiate");
  return TL_OK;
}

}  // namespace

extern "C" int tl_batch_create(tl_batch **out, tl_ctx *const *ctxs, int n) {
  if (!out) return TL_ERR_ARG;
  *out = nullptr;
  tl_batch *b = new (std::nothrow) tl_batch();
  if (!b) return TL_ERR_NOMEM;
  *out = b;
  if (!ctxs || n < 1 || n > BATCH_MAX) {
    snprintf(b->msg, sizeof b->msg, "batch of %d decks outside 1..%d", n, BATCH_MAX);
    return TL_ERR_ARG;
  }
  BCK(cudaGetDevice(&b->device));
  int sms = 0;
  BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
  std::vector<DeckDesc> h(n);
  for (int k = 0; k < n; ++k) {
    tl_ctx *c = ctxs[k];
    if (!c || c->cfg.mode != TL_MODE_TEALEAF || c->device != b->device) {
      snprintf(b->msg, sizeof b->msg, "deck %d: needs a tealeaf-mode context on the current device", k);
      return TL_ERR_ARG;
    }
    b->ctx.push_back(c);
    h[k].F = c->F;
    h[k].g = c->g;
    h[k].ntx = (c->g.nx + 63) / 64;
    h[k].tiles = h[k].ntx * ((c->g.ny + BATCH_ROWS - 1) / BATCH_ROWS);
    h[k].cells = (long long)c->g.nx * c->g.ny;
  }
  // blocks: the occupancy of each batched kernel at 256 threads, at least one per deck
  int occ_w = 0, occ_u = 0;
  BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_w, k_batch_w, 256, 0));
  BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_u, k_batch_ur, 256, 0));
  b->total_w = (occ_w > 0 ? occ_w : 1) * sms;
  b->total_u = (occ_u > 0 ? occ_u : 1) * sms;
  const int maxb = ctxs[0]->max_blocks;
  for (int k = 0; k < n; ++k)
    if (ctxs[k]->max_blocks < maxb) {
      snprintf(b->msg, sizeof b->msg, "deck %d: reduction scratch smaller than the batch's share", k);
      return TL_ERR_ARG;
    }
  if (b->total_w > maxb) b->total_w = maxb;
  if (b->total_u > maxb) b->total_u = maxb;
  if (b->total_w < n) b->total_w = n;
  if (b->total_u < n) b->total_u = n;
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BCK(cudaEventCreate(&b->ev0));
  BCK(cudaEventCreate(&b->ev1));
  BCK(cudaMalloc(&b->d_decks, sizeof(DeckDesc) * n));
  BCK(cudaMalloc(&b->d_map, sizeof(BatchMap)));
  BCK(cudaMallocHost(&b->h_map, sizeof(BatchMap)));
  memset(b->h_map, 0, sizeof(BatchMap));
  b->h_map->n = n;
  b->h_map->total_w = b->total_w;
  b->h_map->total_u = b->total_u;
  BCK(cudaMemcpyAsync(b->d_decks, h.data(), sizeof(DeckDesc) * n, cudaMemcpyHostToDevice, b->stream));
  b->h_decks = h;
  BCK(cudaMemcpyAsync(b->d_map, b->h_map, sizeof(BatchMap), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return TL_OK;
}

extern "C" int tl_batch_destroy(tl_batch *b) {
  if (!b) return TL_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->graph_ir) cudaGraphExecDestroy(b->graph_ir);
  if (b->d_decks) cudaFree(b->d_decks);
  if (b->d_map) cudaFree(b->d_map);
  if (b->h_map) cudaFreeHost(b->h_map);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return TL_OK;
}

extern "C" const char *tl_batch_last_error(const tl_batch *b) { return b ? b->msg : "null batch"; }

namespace {

int grid_cells_of(const Geom &g, int full) {
  long long n = full ? (long long)g.X * g.Y : (long long)g.nx * g.ny;
  long long blocks = (n + 255) / 256;
  if (blocks > 152LL * 32) blocks = 152LL * 32;
  return (int)(blocks < 1 ? 1 : blocks);
}

// The FP32-refined batch: per deck tea_leaf_init (reference operation order),
// copyu!, the FP32 copies and the first test; one graph launch for the
// inner iterations and refinements of every deck; per deck the last search
// direction back to FP64 and the halo of u, p.
int batch_solve_ir(tl_batch *b, const double *rx, const double *ry, const tl_params *prm, tl_result *results) {
  const int n = (int)b->ctx.size();
  for (int k = 0; k < n; ++k) {
    tl_ctx *ctx = b->ctx[k];
    if (!ctx->initialised || prm->maxiters > ctx->cfg.maxiters) {
      snprintf(b->msg, sizeof b->msg, "deck %d: not initialised, or maxiters beyond its tables", k);
      return TL_ERR_STATE;
    }
    const int rc = tl_ensure_ir(ctx, 0);  // the batch walks its own tiles: no single-deck tuning
    if (rc) {
      snprintf(b->msg, sizeof b->msg, "deck %d: %s", k, ctx->msg);
      return rc;
    }
  }
  if (!b->ir_ready) {
    for (int k = 0; k < n; ++k) {
      tl_ctx *ctx = b->ctx[k];
      DeckDesc &D = b->h_decks[k];
      D.g32.nx = ctx->g.nx;
      D.g32.ny = ctx->g.ny;
      D.g32.hd = ctx->g.hd;
      D.g32.X = ctx->g.X;
      D.g32.Y = ctx->g.Y;
      D.g32.pitch = ctx->ir->pitch;
      D.q.r = ctx->ir->r;
      D.q.x = ctx->ir->x;
      D.q.iw = ctx->ir->iw;
      D.p32 = ctx->ir->p;
      D.pb32 = ctx->ir->pb;
      D.ntx32 = (ctx->g.nx + 127) / 128;
      D.tiles32 = D.ntx32 * ((ctx->g.ny + BATCH_ROWS32 - 1) / BATCH_ROWS32);
    }
    BCK(cudaMemcpyAsync(b->d_decks, b->h_decks.data(), sizeof(DeckDesc) * n, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->ir_ready = 1;
  }
  std::vector<cudaStream_t> own(n);
  for (int k = 0; k < n; ++k) {
    own[k] = b->ctx[k]->stream;
    b->ctx[k]->stream = b->stream;
  }
  auto restore = [&]() {
    for (int k = 0; k < n; ++k) b->ctx[k]->stream = own[k];
  };
  tl_params p = *prm;
  p.criterion = TL_CRIT_RELATIVE;
  int rc = TL_OK;
  for (int k = 0; k < n && !rc; ++k) {
    tl_ctx *ctx = b->ctx[k];
    const DeckDesc &D = b->h_decks[k];
    memset(&results[k], 0, sizeof(tl_result));
    results[k].r0_plain = results[k].r0_pred = -1.0;
    ctx->launches = 0;
    rc = tl_cg_init(ctx, rx[k], ry[k], p.coefficient, 1);
    if (!rc) rc = tl_set_loop_params(ctx, &p, 0, 0);
    const int up[2] = {TL_EX_U, TL_EX_P};
    if (!rc) rc = tl_halo_update(ctx, 1, up, 2, 1);
    if (!rc) rc = tl_copy_u(ctx);
    if (!rc) {
      k_ir_convert<<<grid_cells_of(ctx->g, 1), 256, 0, b->stream>>>(ctx->F, ctx->g, D.g32, D.q.r, D.p32, D.q.x);
      k_ir_convert_iw<<<grid_cells_of(ctx->g, 1), 256, 0, b->stream>>>(ctx->F, ctx->g, D.g32, D.q.iw, p.coefficient,
                                                                       rx[k], ry[k]);
      k_batch_ir_start<<<1, 1, 0, b->stream>>>(ctx->F.sc, IR_DELTA * IR_DELTA);
      if (cudaGetLastError() != cudaSuccess) rc = TL_ERR_CUDA;
    }
    if (rc) snprintf(b->msg, sizeof b->msg, "deck %d: %s", k, ctx->msg);
  }
  if (rc) {
    restore();
    return rc;
  }
  k_batch_map<<<1, 256, 0, b->stream>>>(b->d_decks, b->d_map, 0, 0, 1);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !b->graph_ir) rc = build_graph(b, 1);
  if (e == cudaSuccess && !rc) e = cudaEventRecord(b->ev0, b->stream);
  if (e == cudaSuccess && !rc) rc = run_loop(b, 1);
  if (e == cudaSuccess && !rc) e = cudaEventRecord(b->ev1, b->stream);
  if (e == cudaSuccess && !rc) e = cudaEventSynchronize(b->ev1);
  float ms = 0.f;
  if (e == cudaSuccess && !rc) e = cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  b->last_ms = ms;
  if (e != cudaSuccess) rc = bfail(b, e, "FP32-refined batch loop");
  for (int k = 0; k < n && !rc; ++k) {
    tl_ctx *ctx = b->ctx[k];
    const DeckDesc &D = b->h_decks[k];
    k_ir_export_p<<<grid_cells_of(ctx->g, 0), 256, 0, b->stream>>>(ctx->F, ctx->g, D.g32, D.p32);
    const int up[2] = {TL_EX_U, TL_EX_P};
    rc = tl_halo_update(ctx, 1, up, 2, 1);
    if (!rc) rc = tl_read_scalars(ctx);
    if (rc) break;
    const DevScalars &sc = *ctx->host_sc;
    results[k].iters = sc.iter;
    results[k].cg_iters = sc.iter;
    results[k].error = sc.red[0];
    results[k].rel_residual = sc.red[1];
    results[k].converged = sc.converged;
    results[k].refinements = sc.refinements;
    results[k].launches = 0;
  }
  if (!rc) {
    e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) rc = bfail(b, e, "batch epilogue");
  }
  restore();
  return rc;
}

}  // namespace

extern "C" int tl_batch_solve(tl_batch *b, const double *rx, const double *ry, const tl_params *prm,
                              tl_result *results) {
  if (!b || !rx || !ry || !prm || !results) return TL_ERR_ARG;
  if (prm->solver != TL_SOLVER_CG || prm->exact ||
      (prm->precision != TL_PREC_FP64 && prm->precision != TL_PREC_FP32_IR)) {
    snprintf(b->msg, sizeof b->msg, "batched solves run CG (fused FP64 or FP32-refined, exact 0)");
    return TL_ERR_ARG;
  }
  if (prm->precision == TL_PREC_FP32_IR) return batch_solve_ir(b, rx, ry, prm, results);
  const int n = (int)b->ctx.size();
  // each deck's CG.init!, halo of u, p and copyu, on the batch stream
  std::vector<cudaStream_t> own(n);
  for (int k = 0; k < n; ++k) {
    tl_ctx *ctx = b->ctx[k];
    if (!ctx->initialised || prm->maxiters > ctx->cfg.maxiters) {
      snprintf(b->msg, sizeof b->msg, "deck %d: not initialised, or maxiters beyond its tables", k);
      return TL_ERR_STATE;
    }
    own[k] = ctx->stream;
    ctx->stream = b->stream;
  }
  auto restore = [&]() {
    for (int k = 0; k < n; ++k) b->ctx[k]->stream = own[k];
  };
  int rc = TL_OK;
  for (int k = 0; k < n && !rc; ++k) {
    tl_ctx *ctx = b->ctx[k];
    memset(&results[k], 0, sizeof(tl_result));
    ctx->launches = 0;
    rc = tl_cg_init(ctx, rx[k], ry[k], prm->coefficient, 0);
    if (!rc) rc = tl_set_loop_params(ctx, prm, 0, 0);
    const int up[2] = {TL_EX_U, TL_EX_P};
    if (!rc) rc = tl_halo_update(ctx, 1, up, 2, 1);
    if (!rc) rc = tl_copy_u(ctx);
    if (rc) snprintf(b->msg, sizeof b->msg, "deck %d: %s", k, ctx->msg);
  }
  if (rc) {
    restore();
    return rc;
  }
  if (prm->maxiters >= 1) {
    k_batch_map<<<1, 256, 0, b->stream>>>(b->d_decks, b->d_map, 0, 0, 0);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && !b->graph) rc = build_graph(b, 0);
    if (e == cudaSuccess && !rc) e = cudaEventRecord(b->ev0, b->stream);
    if (e == cudaSuccess && !rc) rc = run_loop(b, 0);
    if (e == cudaSuccess && !rc) e = cudaEventRecord(b->ev1, b->stream);
    if (e == cudaSuccess && !rc) e = cudaEventSynchronize(b->ev1);
    float ms = 0.f;
    if (e == cudaSuccess && !rc) e = cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms;
    if (e != cudaSuccess) rc = bfail(b, e, "batch loop");
  }
  // per deck: the last iteration's p! and the halo of u, p; under the
  // relative criterion the true residual u0 - A u measured as in the
  // single-deck solve (the deck counts as converged only if it meets eps);
  // the results
  for (int k = 0; k < n && !rc; ++k) {
    tl_ctx *ctx = b->ctx[k];
    rc = tl_read_scalars(ctx);
    if (rc) break;
    const int iters = ctx->host_sc->iter, conv = ctx->host_sc->converged;
    const double err = ctx->host_sc->error, bb = ctx->host_sc->bb;
    if (prm->maxiters >= 1) {
      const double *pcur = (iters & 1) ? ctx->F.pb : ctx->F.p;
      launch_tl_p(ctx->stream, ctx->F, ctx->g, ctx->walk_ur64, pcur, ctx->F.p, 0);
      rc = tl_halo_update(ctx, 1, nullptr, -1, 1);
    }
    double rel = -1.0;
    if (!rc && prm->criterion == TL_CRIT_RELATIVE) {
      launch_true_resid(ctx->stream, ctx->F, ctx->g, ctx->walk_exact, TL_MODE_TEALEAF, 0);
      if ((rc = tl_read_scalars(ctx))) break;
      const double tr = ctx->host_sc->red[0];
      rel = bb > 0 ? sqrt(tr / bb) : sqrt(tr);
    }
    results[k].iters = iters;
    results[k].cg_iters = iters;
    results[k].error = prm->maxiters >= 1 ? err : ERROR_START;
    results[k].converged = prm->criterion == TL_CRIT_RELATIVE ? (rel >= 0 && rel < prm->eps) : conv;
    results[k].rel_residual = rel;
    results[k].launches = 0;
  }
  if (!rc) {
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) rc = bfail(b, e, "batch epilogue");
  }
  restore();
  return rc;
}

extern "C" int tl_batch_last_ms(tl_batch *b, double *ms) {
  if (!b || !ms) return TL_ERR_ARG;
  *ms = b->last_ms;
  return TL_OK;
}
