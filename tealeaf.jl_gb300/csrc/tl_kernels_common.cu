// tl_kernels_common.cu -- state fill, halo, tea_leaf_init, copyu, residual,
// finalise and field summary kernels.  Every arithmetic step uses explicitly
// rounded double operations (no FMA contraction) in the reference's order, so
// these kernels are bit-identical to the CPU restatement of the reference.
#include "tl_march.cuh"

namespace tl {

// ---------------------------------------------------------------------------
// elementwise helpers over the full (X, Y) array
// ---------------------------------------------------------------------------

__global__ void k_fill(double *f, Geom g, double v) {
  const long long n = (long long)g.X * g.Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(k % g.X), J = (int)(k / g.X);
    f[g.full(I, J)] = v;
  }
}

static inline int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152LL * 32) b = 152LL * 32;
  if (b < 1) b = 1;
  return (int)b;
}

void launch_fill(cudaStream_t st, double *f, const Geom &g, double v) {
  k_fill<<<grid_for((long long)g.X * g.Y, 256), 256, 0, st>>>(f, g, v);
}

__global__ void k_copy_full(double *dst, const double *src, Geom g) {
  const long long n = (long long)g.X * g.Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(k % g.X), J = (int)(k / g.X);
    dst[g.full(I, J)] = src[g.full(I, J)];
  }
}

void launch_copy_full(cudaStream_t st, double *dst, const double *src, const Geom &g) {
  k_copy_full<<<grid_for((long long)g.X * g.Y, 256), 256, 0, st>>>(dst, src, g);
}

// ---------------------------------------------------------------------------
// setchunkstate! (src/chunk.jl:122-151)
// ---------------------------------------------------------------------------

__device__ __forceinline__ double vertex(double lo, double d, int k, int hd) {
  return dadd(lo, dmul(d, (double)(k - hd)));  // chunk.jl:76-77
}

__global__ void k_set_states(Fields F, Geom g, StateTable t, double xmin, double ymin, double dx, double dy,
                             int mode) {
  const long long n = (long long)g.X * g.Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(k % g.X), J = (int)(k / g.X);
    // Reference mode writes energy0[j, k] with j the y-vertex index on
    // dimension 1 (chunk.jl:143-144): memory cell (I, J) holds the test of
    // x-vertex J and y-vertex I.  Tealeaf mode: x-vertex I, y-vertex J.
    const int kx = (mode == TL_MODE_REFERENCE) ? J : I;
    const int jy = (mode == TL_MODE_REFERENCE) ? I : J;
    const double vx0 = vertex(xmin, dx, kx, g.hd), vx1 = vertex(xmin, dx, kx + 1, g.hd);
    const double vy0 = vertex(ymin, dy, jy, g.hd), vy1 = vertex(ymin, dy, jy + 1, g.hd);
    double e = t.s[0].energy, d = t.s[0].density;
    for (int s = 0; s < t.n; ++s) {
      const tl_state &S = t.s[s];
      // Reference mode: every state takes the rectangle arm (Match.jl binds
      // the bare `Rectangular` pattern in chunk.jl:132 as a variable).
      const int geom = (mode == TL_MODE_REFERENCE) ? TL_GEOM_RECTANGULAR : S.geometry;
      bool apply;
      if (geom == TL_GEOM_RECTANGULAR) {
        apply = vx1 >= S.xmin && vx0 < S.xmax && vy1 >= S.ymin && vy0 < S.ymax;
      } else if (geom == TL_GEOM_CIRCULAR) {
        const double cx = dmul(0.5, dadd(vx0, vx1)), cy = dmul(0.5, dadd(vy0, vy1));
        const double ddx = dsub(cx, S.xmin), ddy = dsub(cy, S.ymin);
        apply = dadd(dmul(ddx, ddx), dmul(ddy, ddy)) <= dmul(S.radius, S.radius);
      } else {
        apply = vx0 == S.xmin && vy0 == S.ymin;
      }
      if (apply) {
        e = S.energy;
        d = S.density;
      }
    }
    const size_t c = g.full(I, J);
    F.energy0[c] = e;
    F.density[c] = d;
    if (I >= 1 && I < g.X - 1 && J >= 1 && J < g.Y - 1) F.u[c] = dmul(e, d);  // chunk.jl:148-150
  }
}

void launch_set_states(cudaStream_t st, const Fields &F, const Geom &g, const StateTable &t, double xmin, double ymin,
                       double dx, double dy, int mode) {
  k_set_states<<<grid_for((long long)g.X * g.Y, 256), 256, 0, st>>>(F, g, t, xmin, ymin, dx, dy, mode);
}

// ---------------------------------------------------------------------------
// updateface! (src/kernels.jl:191-210)
// ---------------------------------------------------------------------------

struct HaloFields {
  double *f[6];
  int nf;
};

// One thread per (field, face, layer, position).  face_mask selects faces
// (1 left, 2 right, 4 top, 8 bottom).  Reference mode keeps the 1-based index
// math of the Julia transcription (one cell off a reflection); tealeaf mode
// reflects.  Faces span the interior range of the other axis.
__global__ void k_halo(HaloFields hf, Geom g, int depth, int mode, int face_mask) {
  const int X = g.X, Y = g.Y, hd = g.hd;
  const long long nlr = (long long)depth * g.ny, ntb = (long long)depth * g.nx;
  const long long per_field = 2 * nlr + 2 * ntb;
  const long long n = per_field * hf.nf;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    double *b = hf.f[k / per_field];
    long long q = k % per_field;
    int face;
    if (q < nlr) face = 0;
    else if ((q -= nlr) < nlr) face = 1;
    else if ((q -= nlr) < ntb) face = 2;
    else { q -= ntb; face = 3; }
    if (!(face_mask & (1 << face))) continue;
    const int len = (face < 2) ? g.ny : g.nx;
    const int layer = (int)(q / len);  // 0 .. depth-1
    const int pos = hd + (int)(q % len);
    int dI, dJ, sI, sJ;
    if (mode == TL_MODE_REFERENCE) {
      const int kk = layer + 1;
      switch (face) {
        case 0: dI = hd - kk - 1; sI = hd + kk - 1; dJ = sJ = pos; break;
        case 1: dI = X - hd + kk - 1; sI = X - hd - 2 - kk; dJ = sJ = pos; break;
        case 2: dJ = Y - hd + kk - 1; sJ = Y - hd - 2 - kk; dI = sI = pos; break;
        default: dJ = hd - kk - 1; sJ = hd + kk - 1; dI = sI = pos; break;
      }
    } else {
      const int kk = layer;
      switch (face) {
        case 0: dI = hd - 1 - kk; sI = hd + kk; dJ = sJ = pos; break;
        case 1: dI = X - hd + kk; sI = X - hd - 1 - kk; dJ = sJ = pos; break;
        case 2: dJ = Y - hd + kk; sJ = Y - hd - 1 - kk; dI = sI = pos; break;
        default: dJ = hd - 1 - kk; sJ = hd + kk; dI = sI = pos; break;
      }
    }
    b[g.full(dI, dJ)] = b[g.full(sI, sJ)];
  }
}

void launch_halo(cudaStream_t st, double *const *fields, int nf, const Geom &g, int depth, int mode) {
  if (nf <= 0) return;
  HaloFields hf{};
  for (int k = 0; k < nf; ++k) hf.f[k] = fields[k];
  hf.nf = nf;
  const long long n = (2LL * depth * g.ny + 2LL * depth * g.nx) * nf;
  const int blocks = grid_for(n, 256);
  // The faces read interior cells only when the interior is wider than the
  // update reaches; on tiny grids the reference's face order (left, right,
  // top, bottom) is kept by one launch per face.
  if (g.nx > depth + 1 && g.ny > depth + 1) {
    k_halo<<<blocks, 256, 0, st>>>(hf, g, depth, mode, 15);
  } else {
    for (int f = 0; f < 4; ++f) k_halo<<<blocks, 256, 0, st>>>(hf, g, depth, mode, 1 << f);
  }
}

// ---------------------------------------------------------------------------
// tea_leaf_init (src/solvers/CG.jl:47-79, src/solvers/Jacobi.jl:33-57)
// ---------------------------------------------------------------------------

// u = energy*density, p = r = 0 on the whole array; w = density^(+-1) on halo(1).
// CG.init! (CG.jl:53-60): u = energy * density, p = r = 0, w = density^(+-1)
// on 2:X-1 x 2:Y-1.  With halo depth 1 that range leaves w = 0 in the outer
// halo layer and Kx, Ky at the domain edge infinite; tealeaf mode (w0 = 0)
// computes w over the whole array, which changes nothing for depth >= 2.
__global__ void k_init_pre(Fields F, Geom g, int coefficient, int w0) {
  const long long n = (long long)g.X * g.Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(k % g.X), J = (int)(k / g.X);
    const size_t c = g.full(I, J);
    const double rho = F.density[c];
    F.u[c] = dmul(F.energy[c], rho);
    F.p[c] = 0.0;
    F.r[c] = 0.0;
    if (I >= w0 && I < g.X - w0 && J >= w0 && J < g.Y - w0)
      F.w[c] = (coefficient == TL_CONDUCTIVITY) ? rho : ddiv(1.0, rho);
  }
}

void launch_init_pre(cudaStream_t st, const Fields &F, const Geom &g, int coefficient, int mode) {
  k_init_pre<<<grid_for((long long)g.X * g.Y, 256), 256, 0, st>>>(F, g, coefficient,
                                                                   mode == TL_MODE_TEALEAF ? 0 : 1);
}

// kx, ky over [hd, X-1) x [hd, Y-1): rx*(wl + wc)/(2*wl*wc).  from_density
// takes the coefficient straight from density (Jacobi.jl:44-51).
__global__ void k_init_coef(Fields F, Geom g, double rx, double ry, int from_density, int coefficient) {
  const int W = g.X - 1 - g.hd, H = g.Y - 1 - g.hd;
  const long long n = (long long)W * H;
  const bool recip = coefficient != TL_CONDUCTIVITY;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = g.hd + (int)(k % W), J = g.hd + (int)(k / W);
    const size_t c = g.full(I, J);
    double wc, wl, wd;
    if (from_density) {
      wc = F.density[c];
      wl = F.density[c - 1];
      wd = F.density[c - g.pitch];
      if (recip) {
        wc = ddiv(1.0, wc);
        wl = ddiv(1.0, wl);
        wd = ddiv(1.0, wd);
      }
    } else {
      wc = F.w[c];
      wl = F.w[c - 1];
      wd = F.w[c - g.pitch];
    }
    F.kx[c] = ddiv(dmul(rx, dadd(wl, wc)), dmul(dmul(2.0, wl), wc));
    F.ky[c] = ddiv(dmul(ry, dadd(wd, wc)), dmul(dmul(2.0, wd), wc));
  }
}

void launch_init_coef(cudaStream_t st, const Fields &F, const Geom &g, double rx, double ry, int from_density,
                      int coefficient) {
  const long long n = (long long)(g.X - 1 - g.hd) * (g.Y - 1 - g.hd);
  if (n <= 0) return;
  k_init_coef<<<grid_for(n, 256), 256, 0, st>>>(F, g, rx, ry, from_density, coefficient);
}

// diag = (((1 + kx[i+1]) + kx[i]) + ky[j+1]) + ky[j]: the reference's consum
// (kernels.jl:180), stored once per solve for the fused kernels.
__global__ void k_init_diag(Fields F, Geom g) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    F.diag[c] = dadd(dadd(dadd(dadd(1.0, F.kx[c + 1]), F.kx[c]), F.ky[c + g.pitch]), F.ky[c]);
  }
}

void launch_init_diag(cudaStream_t st, const Fields &F, const Geom &g) {
  k_init_diag<<<grid_for((long long)g.nx * g.ny, 256), 256, 0, st>>>(F, g);
}

// Interior: w = A u, r = u - w, p = r, rro = sum r^2 (CG.jl:70-78).
struct OpInitResid : NoSkip {
  Fields F;
  Geom g;
  int mode;
  __device__ void cell(int i, int j, double (&acc)[1]) const {
    const size_t c = g.at(i, j);
    const double wv = smvp_exact(F, g, F.u, c, mode);
    F.w[c] = wv;
    const double rv = dsub(F.u[c], wv);
    F.r[c] = rv;
    F.p[c] = rv;
    acc[0] = dadd(acc[0], dmul(rv, rv));
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) cell(i0, j, acc);
      if (i0 + 1 < g.nx) cell(i0 + 1, j, acc);
    }
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    sc->rro = tot[0];
    sc->error = ERROR_START;
    sc->iter = 0;
    sc->done = 0;
    sc->converged = 0;
    sc->switched = 0;
    sc->beta = 0.0;
    sc->first = 1;
  }
};

void launch_init_resid(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, int mode) {
  OpInitResid op;
  op.F = F;
  op.g = g;
  op.mode = mode;
  launch_walk<1>(st, op, wk, g.ny);
}

// copyu! (kernels.jl:217-220): u0 = u on the interior; with_bb also sums u0^2.
struct OpCopyU : NoSkip {
  Fields F;
  Geom g;
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) {
        const size_t c = g.at(i0, j);
        const double v = F.u[c];
        F.u0[c] = v;
        acc[0] = dadd(acc[0], dmul(v, v));
      }
      if (i0 + 1 < g.nx) {
        const size_t c = g.at(i0 + 1, j);
        const double v = F.u[c];
        F.u0[c] = v;
        acc[0] = dadd(acc[0], dmul(v, v));
      }
    }
  }
  __device__ void fin(const double *tot) const { F.sc->bb = tot[0]; }
};

void launch_copyu(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, int with_bb) {
  (void)with_bb;
  OpCopyU op;
  op.F = F;
  op.g = g;
  launch_walk<1>(st, op, wk, g.ny);
}

// residual! (kernels.jl:227-232): r = u0 - A u on the interior.
__global__ void k_residual(Fields F, Geom g, int mode) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    F.r[c] = dsub(F.u0[c], smvp_exact(F, g, F.u, c, mode));
  }
}

void launch_residual(cudaStream_t st, const Fields &F, const Geom &g, int mode) {
  k_residual<<<grid_for((long long)g.nx * g.ny, 256), 256, 0, st>>>(F, g, mode);
}

// finalise! (kernels.jl:239-242): energy = u / density on the interior.
__global__ void k_finalise(Fields F, Geom g) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    F.energy[c] = ddiv(F.u[c], F.density[c]);
  }
}

void launch_finalise(cudaStream_t st, const Fields &F, const Geom &g) {
  k_finalise<<<grid_for((long long)g.nx * g.ny, 256), 256, 0, st>>>(F, g);
}

// fieldsummary (kernels.jl:119-133): vol, mass = vol*rho, ie = mass*energy,
// temp = mass*u summed over the interior.
struct OpSummary : NoSkip {
  Fields F;
  Geom g;
  __device__ void cell(int i, int j, double (&acc)[4]) const {
    const size_t c = g.at(i, j);
    const double vol = F.volume[c];
    const double m = dmul(vol, F.density[c]);
    acc[0] = dadd(acc[0], vol);
    acc[1] = dadd(acc[1], m);
    acc[2] = dadd(acc[2], dmul(m, F.energy[c]));
    acc[3] = dadd(acc[3], dmul(m, F.u[c]));
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[4]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) cell(i0, j, acc);
      if (i0 + 1 < g.nx) cell(i0 + 1, j, acc);
    }
  }
  __device__ void fin(const double *tot) const {
    for (int a = 0; a < 4; ++a) F.sc->red[a] = tot[a];
  }
};

// The true residual t = u0 - A u (reference operation order, halo of u read
// from memory): sum t^2 into red[0]; with `write` also r = t, p = t (the
// restart of a CG whose recursive residual drifted from the true one).
struct OpTrueResid : NoSkip {
  Fields F;
  Geom g;
  int mode, write;
  __device__ void cell(int i, int j, double (&acc)[1]) const {
    const size_t c = g.at(i, j);
    const double t = dsub(F.u0[c], smvp_exact(F, g, F.u, c, mode));
    if (write) {
      F.r[c] = t;
      F.p[c] = t;
    }
    acc[0] = dadd(acc[0], dmul(t, t));
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) cell(i0, j, acc);
      if (i0 + 1 < g.nx) cell(i0 + 1, j, acc);
    }
  }
  __device__ void fin(const double *tot) const {
    F.sc->red[0] = tot[0];
    if (write) {
      F.sc->rro = tot[0];
      F.sc->first = 1;
      F.sc->done = 0;
    }
  }
};

void launch_true_resid(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, int mode, int write) {
  OpTrueResid op;
  op.F = F;
  op.g = g;
  op.mode = mode;
  op.write = write;
  launch_walk<1>(st, op, wk, g.ny);
}

void launch_summary(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk) {
  OpSummary op;
  op.F = F;
  op.g = g;
  launch_walk<4>(st, op, wk, g.ny);
}

}  // namespace tl
