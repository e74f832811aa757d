// tl_internal.cuh -- shared definitions of the GB300 TeaLeaf solve library.
//
// Device layout: every Chunk field (src/chunk.jl:24-38) is one pitched 2-D
// array in HBM.  Element (I, J) of the reference's column-major (X, Y) array
// (0-based, I along the contiguous dimension) lives at base[I + J*pitch].
// pitch is a multiple of 16 doubles and each field base is offset by `lead`
// doubles so that the first interior element of every row (I = halodepth) is
// 128-byte aligned: interior column pairs are then 16-byte aligned for double2
// loads.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tealeaf_gb300.h"

namespace tl {

constexpr double ERROR_START = 1e10;      // src/kernels.jl:7
constexpr double ERROR_SWITCH_MAX = 1.0;  // src/kernels.jl:8
constexpr int CGEIGENITERS = 20;          // src/solvers/Cheby.jl:7
constexpr int MAX_STATES = 64;
constexpr int MAX_RED = 4;                // accumulators one reduction kernel can carry

// Geometry of the device arrays.
struct Geom {
  int nx, ny, hd, X, Y;
  long long pitch;  // elements between consecutive columns J (rows of the pitched array)
  __host__ __device__ __forceinline__ size_t at(int i, int j) const {   // interior-relative cell
    return (size_t)(hd + i) + (size_t)(hd + j) * (size_t)pitch;
  }
  __host__ __device__ __forceinline__ size_t full(int I, int J) const {  // full-array index
    return (size_t)I + (size_t)J * (size_t)pitch;
  }
};

// Tile walk of the reduction kernels: tiles of (64*warps) columns x rows
// interior cells, tile t -> (t % ntx, t / ntx), block b walks tiles b, b+G, ...
// Lane l of warp w owns the column pair i0 = 64*w + 2*l of each tile.
struct Walk {
  int warps, rows, blocks, ntx, tiles;
};

// Scalars of a solve, resident in device memory so that the iteration loop
// runs inside a CUDA graph with no host round trip.
struct DevScalars {
  // loop state
  double rro, pw, alpha, beta, rrn, error, bb, theta;
  double red[MAX_RED];  // outputs of plain reductions (summary, norms)
  int iter;             // completed iterations of the current loop
  int done;             // the loop has ended (converged, switched or capped)
  int converged;
  int switched;         // Cheby/PPCG switch condition met
  // parameters read by the loop epilogues
  double eps, epslim;
  int maxiters, presteps, errorswitch, stale_rro, crit, switch_rule;
  int iter_base;        // 1-based loop index of this loop's first trip minus 1
  int cheby_iters, est_iters, calc_every;  // Chebyshev loop bookkeeping
  int first;            // the next fused CG step starts from p itself (no beta update)
  double rr_ref;        // FP32 refinement: r.r at the last refinement
  double delta2;        // FP32 refinement: refine once r.r < delta2 * rr_ref
  // batched FP32 refinement (tl_batch.cu)
  int pbuf;             // 1: the current FP32 search direction is in the second buffer
  int finished;         // the deck's solve is over (converged or out of iterations)
  int refinements;      // FP64 refinement steps taken
  int prestep_switch;   // FP32 CG presteps of Chebyshev: the switch test held (Cheby.jl:25-29)
  double rxh, ryh;      // FP32 stencil from inverse weights: Kx = rxh (iw_l + iw_c), Ky = ryh (iw_d + iw_c)
};

// Device pointers of one context, passed to kernels by value.
struct Fields {
  double *density0, *density, *energy0, *energy, *u, *u0, *p, *r, *mi, *w, *kx, *ky, *sd, *volume;
  double *pb;    // second p buffer (ping-pong of the fused CG step)
  double *ub;    // second u buffer (Chebyshev step)
  double *sdb;   // second sd buffer (PPCG inner step)
  double *diag;  // 1 + kx[i+1] + kx[i] + ky[j+1] + ky[j] for the fused kernels
  double *cgalpha, *cgbeta, *chebyalpha, *chebybeta;
  DevScalars *sc;
  double *partials;   // reduction scratch: MAX_RED * blocks doubles
  unsigned *counter;  // last-block ticket
};

struct StateTable {
  tl_state s[MAX_STATES];
  int n;
};

// ---- launchers (defined in the .cu files) --------------------------------
void launch_fill(cudaStream_t st, double *f, const Geom &g, double v);
void launch_set_states(cudaStream_t st, const Fields &F, const Geom &g, const StateTable &t, double xmin,
                       double ymin, double dx, double dy, int mode);
void launch_copy_full(cudaStream_t st, double *dst, const double *src, const Geom &g);
// halo of up to 6 fields; `fields` holds device pointers
void launch_halo(cudaStream_t st, double *const *fields, int nf, const Geom &g, int depth, int mode);

void launch_init_pre(cudaStream_t st, const Fields &F, const Geom &g, int coefficient, int mode);
void launch_init_coef(cudaStream_t st, const Fields &F, const Geom &g, double rx, double ry, int from_density,
                      int coefficient);
void launch_init_diag(cudaStream_t st, const Fields &F, const Geom &g);
void launch_init_resid(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, int mode);
void launch_copyu(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, int with_bb);
void launch_residual(cudaStream_t st, const Fields &F, const Geom &g, int mode);
void launch_finalise(cudaStream_t st, const Fields &F, const Geom &g);
void launch_summary(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk);
void launch_true_resid(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, int mode, int write);

// CG iteration kernels.  `cond` is the while-node handle (0 when not in a graph).
void launch_ref_w(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk);
void launch_ref_ur(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, cudaGraphConditionalHandle cond,
                   int set_cond);
void launch_ref_p(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk);
void launch_tl_w(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *psrc, double *pdst,
                 int exact, int guard, int store_coef = 1);
void launch_tl_ur(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *p, int exact,
                  int guard, cudaGraphConditionalHandle cond, int set_cond);
void launch_tl_p(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *psrc, double *pdst,
                 int exact);

// Chebyshev, PPCG and Jacobi kernels (tl_kernels_cheby.cu)
void launch_cheby_init(cudaStream_t st, const Fields &F, const Geom &g, double theta);
void launch_cheby_step(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *usrc,
                       double *udst, int exact, int guard, int force_norm, cudaGraphConditionalHandle cond,
                       int set_cond);
void launch_ppcg_ur(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *p, double *sd,
                    int exact, int guard);
void launch_ppcg_inner(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *sdsrc,
                       double *sddst, int pp, int last, int exact, int guard, cudaGraphConditionalHandle cond,
                       int set_cond);
void launch_jacobi(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *usrc, double *udst,
                   int guard, int exact);
void launch_init_rdiag(cudaStream_t st, const Fields &F, const Geom &g);  // diag = 1 / (1 + sum k)
void launch_jacobi_check(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *u, int guard,
                         cudaGraphConditionalHandle cond, int set_cond);
void launch_norm_r(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk);
void launch_ppcg_sd_final(cudaStream_t st, const Fields &F, const Geom &g, const double *fin, const double *prev);
void launch_copy_interior(cudaStream_t st, double *dst, const double *src, const Geom &g);

}  // namespace tl
