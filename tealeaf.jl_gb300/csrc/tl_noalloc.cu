// tl_noalloc.cu -- the field summary of caller-owned device arrays with no
// device allocation by the library (tl_field_summary_noalloc).
//
// The summary's two-pass reduction needs scratch memory for the block
// partials and the last-block ticket.  Here that scratch is a file-scope
// __device__ array, not memory obtained from cudaMalloc: every GPU that loads
// this library holds one copy (about 33 KB) until the process exits, and every
// call on that GPU shares it.
//
// Host code cannot use the array's name as a device address, so the address
// is looked up with cudaGetSymbolAddress, with the device current, the first
// time a call runs in a device context.  The lookup is keyed on the context's
// id: after cudaDeviceReset the primary context is created again, the module
// is loaded again and the array may move, so a call in the new context looks
// the address up again instead of writing through a stale one.
#include <cstdio>
#include <mutex>

#include <cuda.h>

#include "tl_walk.cuh"

namespace {

constexpr int NOALLOC_MAX_BLOCKS = 1024;                                 // block partials the scratch holds
constexpr int NOALLOC_SCRATCH = tl::MAX_RED * NOALLOC_MAX_BLOCKS + 32;  // + the ticket, in doubles
constexpr long long NOALLOC_MAX_CELLS = 2147483647LL;                    // interior cells per call
// Per-dimension limits: the tile walk forms column and row indices, tile
// counts and hd + i in int, so xcells + 2*halodepth plus one tile width (256
// columns) and ycells + 2*halodepth plus one tile height (8 rows) must stay
// below INT_MAX.  These bounds keep every such sum far from it.
constexpr int NOALLOC_MAX_DIM = 1 << 30;                                 // xcells, ycells
constexpr int NOALLOC_MAX_HALO = 1 << 20;                                // halodepth
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH];

std::mutex g_setup_mutex;
double *g_scratch_addr[MAX_DEVICES];
unsigned long long g_scratch_ctx[MAX_DEVICES];  // id of the context the address was looked up in
int g_sm_count[MAX_DEVICES];

// cuCtxGetCurrent and cuCtxGetId through the runtime's driver entry points
// (the library links the static runtime, not libcuda).
typedef CUresult (*PFN_ctxGetCurrent)(CUcontext *);
typedef CUresult (*PFN_ctxGetId)(CUcontext, unsigned long long *);
PFN_ctxGetCurrent g_ctx_get_current;
PFN_ctxGetId g_ctx_get_id;

// Id of the current context, 0 when there is none; the caller holds the mutex.
unsigned long long current_context_id() {
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || !f1 ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q2 != cudaDriverEntryPointSuccess || !f2)
      return 0;
    g_ctx_get_current = reinterpret_cast<PFN_ctxGetCurrent>(f1);
    g_ctx_get_id = reinterpret_cast<PFN_ctxGetId>(f2);
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c || g_ctx_get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// vol, mass = vol*rho, ie = mass*energy, temp = mass*u over the interior, in
// the same order and reduction tree as the context's field summary.
struct OpSummaryNoAlloc : tl::NoSkip {
  tl::Fields F;
  tl::Geom g;
  double *out;
  __device__ void cell(int i, int j, double (&acc)[4]) const {
    const size_t c = g.at(i, j);
    const double vol = F.volume[c];
    const double m = tl::dmul(vol, F.density[c]);
    acc[0] = tl::dadd(acc[0], vol);
    acc[1] = tl::dadd(acc[1], m);
    acc[2] = tl::dadd(acc[2], tl::dmul(m, F.energy[c]));
    acc[3] = tl::dadd(acc[3], tl::dmul(m, F.u[c]));
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[4]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) cell(i0, j, acc);
      if (i0 + 1 < g.nx) cell(i0 + 1, j, acc);
    }
  }
  __device__ void fin(const double *tot) const {
    for (int a = 0; a < 4; ++a) out[a] = tot[a];
  }
};

int fail(char *err, int errlen, int code, const char *msg) {
  if (err && errlen > 0) snprintf(err, (size_t)errlen, "%s", msg);
  return code;
}

}  // namespace

extern "C" int tl_field_summary_noalloc(const double *volume, const double *density, const double *energy,
                                        const double *u, int xcells, int ycells, int halodepth, long long pitch,
                                        double *out, void *stream, char *err, int errlen) {
  if (err && errlen > 0) err[0] = 0;
  if (!volume || !density || !energy || !u || !out)
    return fail(err, errlen, TL_ERR_ARG, "tl_field_summary_noalloc: null array pointer");
  if (xcells < 1 || ycells < 1 || halodepth < 1)
    return fail(err, errlen, TL_ERR_ARG, "tl_field_summary_noalloc: cells and halo depth must be >= 1");
  if (xcells > NOALLOC_MAX_DIM || ycells > NOALLOC_MAX_DIM || halodepth > NOALLOC_MAX_HALO)
    return fail(err, errlen, TL_ERR_ARG,
                "tl_field_summary_noalloc: xcells, ycells above the maximum of 1073741824 per dimension or "
                "halodepth above 1048576");
  if ((long long)xcells * ycells > NOALLOC_MAX_CELLS)
    return fail(err, errlen, TL_ERR_ARG,
                "tl_field_summary_noalloc: xcells*ycells exceeds the maximum of 2147483647 interior cells");
  if (pitch < (long long)xcells + 2LL * halodepth)
    return fail(err, errlen, TL_ERR_ARG, "tl_field_summary_noalloc: pitch is smaller than xcells + 2*halodepth");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
    return fail(err, errlen, TL_ERR_CUDA, "tl_field_summary_noalloc: no usable current device");
  double *scratch = nullptr;
  int sms = 0;
  {
    // First call in this device's current context: look up the device
    // address of the scratch array with this device current.  Host code
    // cannot use the array's name as an address.  A context created again
    // (after cudaDeviceReset) has a new id and gets a new lookup.
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    const unsigned long long ctx = current_context_id();
    if (!ctx) return fail(err, errlen, TL_ERR_CUDA, "tl_field_summary_noalloc: no current device context");
    if (!g_scratch_addr[dev] || g_scratch_ctx[dev] != ctx) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof msg, "tl_field_summary_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return fail(err, errlen, TL_ERR_CUDA, msg);
      }
      int n = 0;
      e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess || n < 1) return fail(err, errlen, TL_ERR_CUDA, "tl_field_summary_noalloc: no SM count");
      g_sm_count[dev] = n;
      g_scratch_addr[dev] = static_cast<double *>(p);
      g_scratch_ctx[dev] = ctx;
    }
    scratch = g_scratch_addr[dev];
    sms = g_sm_count[dev];
  }

  tl::Geom g;
  g.nx = xcells;
  g.ny = ycells;
  g.hd = halodepth;
  g.X = xcells + 2 * halodepth;
  g.Y = ycells + 2 * halodepth;
  g.pitch = pitch;
  // the context's reduction layout: 4 warps, 8 rows per tile, at most 2 blocks per SM
  tl::Walk wk;
  wk.warps = 4;
  wk.rows = 8;
  wk.ntx = (xcells + 255) / 256;
  const long long tiles = (long long)wk.ntx * ((ycells + 7) / 8);
  wk.tiles = (int)tiles;
  long long blocks = tiles < 2LL * sms ? tiles : 2LL * sms;
  if (blocks > NOALLOC_MAX_BLOCKS) blocks = NOALLOC_MAX_BLOCKS;
  wk.blocks = (int)blocks;

  OpSummaryNoAlloc op;
  op.F = tl::Fields{};
  op.F.volume = const_cast<double *>(volume);
  op.F.density = const_cast<double *>(density);
  op.F.energy = const_cast<double *>(energy);
  op.F.u = const_cast<double *>(u);
  op.F.partials = scratch;
  op.F.counter = reinterpret_cast<unsigned *>(scratch + tl::MAX_RED * NOALLOC_MAX_BLOCKS);
  op.g = g;
  op.out = out;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the ticket must start at zero; the partials are overwritten before use
  cudaError_t e = cudaMemsetAsync(op.F.counter, 0, sizeof(unsigned), st);
  if (e == cudaSuccess) {
    tl::launch_walk<4>(st, op, wk, g.ny);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof msg, "tl_field_summary_noalloc: %s", cudaGetErrorString(e));
    return fail(err, errlen, TL_ERR_CUDA, msg);
  }
  return TL_OK;
}
