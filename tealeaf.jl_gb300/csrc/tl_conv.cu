// tl_conv.cu -- kernels of the warm-start network: 3x3 convolutions as
// implicit GEMMs on the BF16 tensor cores (warp-level mma m16n8k16, FP32
// accumulation) for the forward pass, the input gradient and the weight
// gradient; feature assembly; the residual loss through the 5-point operator;
// Adam.
//
// Activations are NHWC BF16 (N images of H rows x W pixels, C = 16 or 32
// channels contiguous per pixel), zero-padded outside each image.  The three
// input channels are padded to 16 and the one output channel to 16.  Weights
// of a layer are [Cout][9][Cin] BF16 (tap = 3*dy + dx), biases FP32.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "tl_conv.h"

namespace {

using bf16 = __nv_bfloat16;
constexpr int TP = 64;  // pixels of one image row per block (4 warps x 16)

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const void *p) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}

__device__ __forceinline__ void ldsm_x2_trans(uint32_t (&r)[2], const void *p) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(s));
}

// GELU, tanh form: 0.5 z (1 + tanh(c (z + 0.044715 z^3))), c = sqrt(2/pi)
__device__ __forceinline__ float gelu(float z) {
  const float c = 0.7978845608028654f;
  return 0.5f * z * (1.f + tanhf(c * (z + 0.044715f * z * z * z)));
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float c = 0.7978845608028654f;
  const float t = tanhf(c * (z + 0.044715f * z * z * z));
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * z * z);
}

struct ConvArgs {
  const bf16 *x, *w, *gz;
  const float *bias;
  bf16 *z, *out;
  float *out32;
  int N, H, W;
};

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}

// 16-byte asynchronous copy global -> shared; `bytes` = 0 writes zeros
// (the source address must still be a valid one).
__device__ __forceinline__ void cp_async16(void *dst, const void *src, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(src), "r"(bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
// Commits this thread's outstanding copies as a group and waits for all of
// them (wait_group alone would not cover copies never committed).
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

constexpr int FTP = 128;  // forward: pixels of one image row per block (4 warps x 32)
constexpr int FRB = 16;   // forward: image rows swept by one block

template <int CIN, int COUT>
constexpr int conv_smem_bytes() {
  return 2 * (COUT * (9 * CIN + 8) + 4 * (FTP + 2) * (CIN + 8));
}

// One block: FTP pixels x FRB rows of one image, all COUT channels; warp w
// owns pixels [32w, 32w+32) (two 16-pixel m-tiles) of the row being
// computed.  The weights stay in shared memory for the whole sweep.  Input
// rows live in a four-slot ring filled by cp.async: row y+2 is fetched while
// row y is computed, and one barrier per row both publishes the new row and
// frees the slot the next fetch overwrites.  K = 9 taps x CIN in steps of 16;
// A (pixels x channels) and B (channels x output channels) fragments come
// from ldmatrix.
// MODE 0: out = z; 1: out = GELU(z) (z stored when `z` is set);
// 2: out = z * GELU'(gz) (input gradient fused with the GELU derivative).
// `out32` (when set) receives channel 0 of z in FP32.
template <int CIN, int COUT, int MODE>
__global__ void __launch_bounds__(128) k_conv3x3(ConvArgs a) {
  constexpr int PS = CIN + 8;      // pixel stride in shared memory (bf16 elements)
  constexpr int WS = 9 * CIN + 8;  // weight row stride
  constexpr int NT = COUT / 8;
  constexpr int V = CIN / 8;       // 16-byte vectors per pixel
  extern __shared__ __align__(16) unsigned char smem_raw[];
  bf16 *sw = reinterpret_cast<bf16 *>(smem_raw);                   // [COUT][WS]
  bf16 *sx = sw + COUT * WS;                                        // [4][FTP + 2][PS]
  const int img = blockIdx.z, x0 = blockIdx.x * FTP, y0 = blockIdx.y * FRB;
  const int y1 = min(a.H, y0 + FRB);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3, px = warp * 32;
  const size_t plane = (size_t)a.H * a.W;
  const bf16 *xi = a.x + (size_t)img * plane * CIN;

  for (int v = tid; v < COUT * 9 * V; v += 128) {
    const int row = v / (9 * V), c = v % (9 * V);
    cp_async16(sw + row * WS + c * 8, a.w + (size_t)v * 8, 16);
  }
  auto load_row = [&](int yy) {
    bf16 *dst = sx + ((yy + 4) & 3) * (FTP + 2) * PS;
    for (int v = tid; v < (FTP + 2) * V; v += 128) {
      const int col = v / V, c8 = v % V, xx = x0 + col - 1;
      const bool in = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
      const bf16 *src = in ? xi + ((size_t)yy * a.W + xx) * CIN + c8 * 8 : xi;
      cp_async16(dst + col * PS + c8 * 8, src, in ? 16 : 0);
    }
  };
  load_row(y0 - 1);
  load_row(y0);
  load_row(y0 + 1);
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  // ldmatrix row addresses: A matrix j = lane/8 covers pixels +8*(j&1), channels +8*(j>>1);
  // B matrix j covers output channels +8*(j>>1), k +8*(j&1)
  const int lj = lane >> 3, lr = lane & 7;
  for (int y = y0; y < y1; ++y) {
    if (y + 2 <= y1) {
      load_row(y + 2);
      cp_async_commit();
    }
    float acc[2][NT][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int n = 0; n < NT; ++n) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.f;
    // MODE 2: the epilogue's GELU' inputs, loaded before the MMAs so that
    // their latency overlaps the math
    __nv_bfloat162 gzr[2][2][MODE == 2 ? NT : 1];
    if (MODE == 2) {
#pragma unroll
      for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          const int xx = x0 + px + 16 * m + g + 8 * half;
          const size_t o = ((size_t)img * plane + (size_t)y * a.W + (xx < a.W ? xx : 0)) * COUT;
#pragma unroll
          for (int n = 0; n < (MODE == 2 ? NT : 1); ++n)
            gzr[m][half][n] = *reinterpret_cast<const __nv_bfloat162 *>(a.gz + o + n * 8 + 2 * t);
        }
    }
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
      const bf16 *srow = sx + ((y - 1 + dy + 4) & 3) * (FTP + 2) * PS;
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        const int tap = 3 * dy + dx;
#pragma unroll
        for (int cc = 0; cc < CIN; cc += 16) {
          uint32_t af[2][4];
#pragma unroll
          for (int m = 0; m < 2; ++m)
            ldsm_x4(af[m], srow + (px + 16 * m + 8 * (lj & 1) + lr + dx) * PS + cc + 8 * (lj >> 1));
#pragma unroll
          for (int n2 = 0; n2 < NT; n2 += 2) {
            uint32_t bq[4];
            ldsm_x4(bq, sw + (n2 * 8 + 8 * (lj >> 1) + lr) * WS + tap * CIN + cc + 8 * (lj & 1));
            const uint32_t b0[2] = {bq[0], bq[1]}, b1[2] = {bq[2], bq[3]};
#pragma unroll
            for (int m = 0; m < 2; ++m) {
              mma_bf16(acc[m][n2], af[m], b0);
              mma_bf16(acc[m][n2 + 1], af[m], b1);
            }
          }
        }
      }
    }
    // rows g and g+8 of each 16-pixel m-tile; channels n*8 + 2t, +1
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int xx = x0 + px + 16 * m + g + 8 * half;
        if (xx >= a.W) continue;
        const size_t pix = (size_t)img * plane + (size_t)y * a.W + xx;
        const size_t o = pix * COUT;
#pragma unroll
        for (int n = 0; n < NT; ++n) {
          const int ch = n * 8 + 2 * t;
          float z0 = acc[m][n][2 * half], z1 = acc[m][n][2 * half + 1];
          if (a.bias) {
            z0 += a.bias[ch];
            z1 += a.bias[ch + 1];
          }
          if (a.out32 && ch == 0) a.out32[pix] = z0;
          float o0 = z0, o1 = z1;
          if (MODE == 1) {
            if (a.z) *reinterpret_cast<__nv_bfloat162 *>(a.z + o + ch) = __floats2bfloat162_rn(z0, z1);
            o0 = gelu(z0);
            o1 = gelu(z1);
          } else if (MODE == 2) {
            const __nv_bfloat162 zz = gzr[m][half][MODE == 2 ? n : 0];
            o0 = z0 * gelu_grad(__low2float(zz));
            o1 = z1 * gelu_grad(__high2float(zz));
          }
          if (a.out) *reinterpret_cast<__nv_bfloat162 *>(a.out + o + ch) = __floats2bfloat162_rn(o0, o1);
        }
      }
    cp_async_wait_all();
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// The same convolution on the 5th-generation tensor cores (tcgen05)
// ---------------------------------------------------------------------------
//
// One block computes FTP = 128 pixels of an image row per step, FRB rows in
// turn, as a GEMM with M = 128 pixels, N = COUT, K = 9 taps x CIN: one
// tcgen05.mma (M 128, N COUT, K 16, BF16 in, FP32 accumulate) per tap and
// 16-channel step, issued by one thread, accumulating in tensor memory.
// Operands are read by the tensor core straight from shared memory through
// matrix descriptors in the no-swizzle K-major layout, whose unit is an 8 x 8
// BF16 core matrix of eight 16-byte rows:
//   input row:  [CIN/8 channel chunks][FTP + 2 pixels][8 channels]; the core
//               matrices of a chunk are 128 B apart along the pixels (SBO) and
//               the chunks (FTP + 2) x 16 B apart (LBO, the K direction), so
//               the A operand of tap (dy, dx) is the staged row y - 1 + dy
//               shifted by dx pixels: a descriptor, no im2col copy;
//   weights:    [9 CIN/8 k chunks][COUT][8 k values]; core matrices 128 B apart
//               along the output channels (SBO), k chunks COUT x 16 B apart (LBO).
// Input rows live in a ring of RING slots filled by cp.async, fetched
// RING - 1 rows ahead of the row being computed.  The MMAs of a row complete on an
// mbarrier (tcgen05.commit); every thread then reads its pixel's COUT
// accumulators from its warp's tensor-memory lane quadrant (tcgen05.ld) for
// the epilogue.  Every mbarrier wait is bounded: a wait that runs out stops
// the block and counts in g_conv_timeouts.
namespace tc {

__device__ int g_conv_timeouts;

// cp.async.wait_group with a run-time count of groups allowed in flight (0..3).
__device__ __forceinline__ void cp_async_wait_pending(int n) {
  switch (n) {
    case 0: asm volatile("cp.async.wait_group 0;\n" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
  }
}
constexpr int RING = 4;  // staged input rows: rows y - 1 .. y + 2 while row y is computed (six measured no faster)

// GELU and its derivative with the hardware tanh (tanh.approx.f32, relative
// error about 2^-11, below the BF16 rounding of the outputs).
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;\n" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_hw(float z) {
  const float c = 0.7978845608028654f;
  return 0.5f * z * (1.f + tanh_hw(c * (z + 0.044715f * z * z * z)));
}
__device__ __forceinline__ float gelu_grad_hw(float z) {
  const float c = 0.7978845608028654f;
  const float t = tanh_hw(c * (z + 0.044715f * z * z * z));
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * z * z);
}
constexpr int SPIN_LIMIT = 1 << 22;
constexpr int TCOLS = 32;  // tensor-memory columns of one accumulator buffer (COUT <= 32); two per block

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: no swizzle, start, leading (K) and stride
// (M/N) byte offsets, descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: F32 accumulator, BF16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t *bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 16 consecutive FP32 accumulator columns of this thread's lane.
__device__ __forceinline__ void tld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// 8 consecutive FP32 accumulator columns of this thread's lane.
__device__ __forceinline__ void tld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

template <int CIN, int COUT>
struct Smem {
  static constexpr int NC = CIN / 8;             // channel chunks of an input pixel
  static constexpr int ROWB = (FTP + 2) * 16;    // bytes of one chunk of a staged row
  static constexpr int SLOT = NC * ROWB;         // bytes of one staged input row
  static constexpr int KC = 9 * CIN / 8;         // k chunks of the weights
  static constexpr int WB = KC * COUT * 16;      // bytes of the weights
  static constexpr int BIAS = WB + RING * SLOT;  // COUT floats
  static constexpr int BAR = BIAS + 4 * COUT;    // two mbarriers and the tensor-memory address
  static constexpr int BYTES = BAR + 32;
};

// Rows are pipelined: while the epilogue of row y reads its accumulators
// from one tensor-memory buffer, the MMAs of row y + 1 run into the other.
// Eight warps: warp w reads the lane quadrant w % 4 (pixels 32 (w % 4) ..
// + 31) and the output-channel half w / 4 of the accumulators.
template <int CIN, int COUT, int MODE>
__global__ void __launch_bounds__(256) k_conv3x3_tc(ConvArgs a) {
  using S = Smem<CIN, COUT>;
  static_assert(COUT % 16 == 0 && COUT <= TCOLS && CIN % 16 == 0, "tile shape");
  constexpr uint32_t ID = idesc(128, COUT);
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sw = smem;
  unsigned char *sx = smem + S::WB;
  float *sbias = reinterpret_cast<float *>(smem + S::BIAS);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + S::BAR);  // bar[0], bar[1]
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 2);
  const int img = blockIdx.z, x0 = blockIdx.x * FTP, y0 = blockIdx.y * FRB;
  const int y1 = min(a.H, y0 + FRB);
  constexpr int NT = 256, CH = COUT / 2;  // threads; output channels per thread
  const int tid = threadIdx.x, warp = tid >> 5, quad = warp & 3, half = warp >> 2;
  const size_t plane = (size_t)a.H * a.W;
  const bf16 *xi = a.x + (size_t)img * plane * CIN;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                 "r"(2 * TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bar + 1)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.f;
  for (int v = tid; v < COUT * S::KC; v += NT) {
    const int co = v / S::KC, kc = v % S::KC;
    cp_async16(sw + (kc * COUT + co) * 16, a.w + (size_t)co * 9 * CIN + kc * 8, 16);
  }
  auto load_row = [&](int yy) {
    unsigned char *dst = sx + ((yy + RING) % RING) * S::SLOT;
    for (int v = tid; v < (FTP + 2) * S::NC; v += NT) {
      const int col = v / S::NC, c8 = v % S::NC, xx = x0 + col - 1;
      const bool in = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
      const bf16 *src = in ? xi + ((size_t)yy * a.W + xx) * CIN + c8 * 8 : xi;
      cp_async16(dst + c8 * S::ROWB + col * 16, src, in ? 16 : 0);
    }
  };
  const uint32_t wbase = saddr(sw), xbase = saddr(sx);
  // the MMAs of row y into tensor-memory buffer b, completing on bar[b]
  auto issue = [&](int y, int b, uint32_t tmem) {
    const uint32_t d = tmem + b * TCOLS;
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
      const uint32_t rbase = xbase + ((y - 1 + dy + RING) % RING) * S::SLOT;
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        const int tap = 3 * dy + dx;
#pragma unroll
        for (int cc = 0; cc < CIN; cc += 16) {
          const uint64_t ad = sdesc(rbase + (cc / 8) * S::ROWB + dx * 16, S::ROWB, 128);
          const uint64_t bd = sdesc(wbase + ((tap * CIN + cc) / 8) * COUT * 16, COUT * 16, 128);
          mma(d, ad, bd, ID, (tap | cc) != 0);
        }
      }
    }
    commit(bar + b);
  };
  // rows y0 - 1 .. y0 + 1 for the first MMAs, then y0 + 2 .. y0 + RING - 2,
  // one group each, in flight
  for (int r = -1; r <= 1; ++r)
    if (y0 + r <= y1) load_row(y0 + r);
  cp_async_commit();
  for (int r = 2; r <= RING - 2; ++r)
    if (y0 + r <= y1) {
      load_row(y0 + r);
      cp_async_commit();
    }
  // the first group (weights, rows y0 - 1 .. y0 + 1) must have landed
  cp_async_wait_pending(min(max(y1 - (y0 + 1), 0), RING - 3));
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  if (tid == 0) issue(y0, 0, tmem);
  uint32_t phases = 0u;  // bit b: the parity of mbarrier b's next completion
  const int xx = x0 + 32 * quad + (tid & 31);  // this thread's pixel in the epilogue
  for (int y = y0; y < y1; ++y) {
    const int b = (y - y0) & 1;
    // MODE 2: the epilogue's GELU' inputs, loaded while the MMAs run
    uint4 gzv[MODE == 2 ? CH / 8 : 1];
    if (MODE == 2 && xx < a.W) {
      const uint4 *gp =
          reinterpret_cast<const uint4 *>(a.gz + ((size_t)img * plane + (size_t)y * a.W + xx) * COUT + half * CH);
#pragma unroll
      for (int q = 0; q < (MODE == 2 ? CH / 8 : 1); ++q) gzv[q] = gp[q];
    }
    bool done = false;
    for (int it = 0; it < SPIN_LIMIT && !done; ++it) done = bar_try(bar + b, (phases >> b) & 1u);
    phases ^= 1u << b;
    if (__syncthreads_or(!done)) {
      if (tid == 0) atomicAdd(&g_conv_timeouts, 1);
      break;
    }
    // the MMAs of row y are done: row y - 1's slot takes row y + RING - 1
    if (y + RING - 1 <= y1) {
      load_row(y + RING - 1);
      cp_async_commit();
    }
    if (y + 1 < y1) {
      // row y + 2 must have landed; the rows after it, up to y + RING - 1, may
      // still be in flight (one group per row)
      cp_async_wait_pending(min(max(y1 - (y + 2), 0), RING - 3));
      fence_async_smem();
      fence_before();
      __syncthreads();
      fence_after();
      if (tid == 0) issue(y + 1, b ^ 1, tmem);
    }
    fence_after();
    float acc[CH];
    {
      const uint32_t ta = tmem + ((uint32_t)(32 * quad) << 16) + b * TCOLS + half * CH;
      if (CH == 16) {
        float v[16];
        tld16(ta, v);
#pragma unroll
        for (int k = 0; k < CH; ++k) acc[k] = v[k];
      } else {
        float v[8];
        tld8(ta, v);
#pragma unroll
        for (int k = 0; k < CH; ++k) acc[k] = v[k];
      }
    }
    fence_before();
    if (xx < a.W) {
      const size_t pix = (size_t)img * plane + (size_t)y * a.W + xx;
#pragma unroll
      for (int c = 0; c < CH; ++c) acc[c] += sbias[half * CH + c];
      if (a.out32 && half == 0) a.out32[pix] = acc[0];
      uint4 zo[CH / 8], oo[CH / 8];
#pragma unroll
      for (int q = 0; q < CH / 8; ++q) {
        __nv_bfloat162 *zp = reinterpret_cast<__nv_bfloat162 *>(&zo[q]);
        __nv_bfloat162 *op = reinterpret_cast<__nv_bfloat162 *>(&oo[q]);
        const __nv_bfloat162 *gq = reinterpret_cast<const __nv_bfloat162 *>(&gzv[MODE == 2 ? q : 0]);
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const float z0 = acc[8 * q + 2 * h], z1 = acc[8 * q + 2 * h + 1];
          float o0 = z0, o1 = z1;
          if (MODE == 1) {
            zp[h] = __floats2bfloat162_rn(z0, z1);
            o0 = gelu_hw(z0);
            o1 = gelu_hw(z1);
          } else if (MODE == 2) {
            o0 = z0 * gelu_grad_hw(__low2float(gq[h]));
            o1 = z1 * gelu_grad_hw(__high2float(gq[h]));
          }
          op[h] = __floats2bfloat162_rn(o0, o1);
        }
      }
      if (MODE == 1 && a.z) {
        uint4 *zd = reinterpret_cast<uint4 *>(a.z + pix * COUT + half * CH);
#pragma unroll
        for (int q = 0; q < CH / 8; ++q) zd[q] = zo[q];
      }
      if (a.out) {
        uint4 *od = reinterpret_cast<uint4 *>(a.out + pix * COUT + half * CH);
#pragma unroll
        for (int q = 0; q < CH / 8; ++q) od[q] = oo[q];
      }
    }
  }
  cp_async_wait_all();
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * TCOLS));
}


// ---------------------------------------------------------------------------
// Warp-specialised, row-streaming form: the same implicit GEMM, with the
// producer, the MMA issuer and the epilogue decoupled by mbarriers.
// ---------------------------------------------------------------------------
//
// A persistent block walks tiles of 128 pixels x th rows (WsWalk; th is
// chosen per launch to balance the blocks' work).  Ten warps:
//   warp 0      producer: stages the input rows y0 - 1 .. y0 + rows of a
//               tile, in turn, in a ring of RING slots;
//   warp 1      MMA issuer (one lane), row streaming: each staged input row is
//               read by the tensor core once per (dx, 16-channel step) with
//               B = the weights of dy = 2, 1, 0 stacked (N = up to 3 COUT),
//               accumulating into the up to three output rows it feeds, which
//               sit in consecutive tensor-memory slots of a ring of NACC; it
//               then frees the input row (`empty`, by tcgen05.commit) and
//               hands the output row that is now complete to the epilogue
//               (`tfull`);
//   warps 2..9  epilogue: wait for `tfull`, read the accumulator (tcgen05.ld;
//               lane quadrant warp % 4, channel half (warp - 2) / 4), release
//               it (`tempty`), then bias, GELU and the stores.
// Rows stream across tile boundaries, so loads, MMAs and epilogues of
// neighbouring rows and tiles overlap.  Every mbarrier wait is bounded: one
// that runs out raises the block's abort flag (every role then leaves its
// loop) and counts in g_conv_timeouts.
//
// Two producers:
//   TMA (the default): one thread issues one cp.async.bulk.tensor load per
//     row (box: CIN channels x 130 pixels, zero-filled outside the image)
//     that completes on the row's `full` mbarrier.  The row lands as 130
//     pixel rows of 2 CIN bytes under the 64-byte (CIN 32) or 32-byte (CIN
//     16) swizzle, which the A descriptors name (K-major, 8-row groups 8 x 2
//     CIN bytes apart); the tap shift dx is a start address 2 CIN dx bytes on
//     and the channel step cc one 2 cc bytes on, the swizzle being a function
//     of the shared-memory address bits.  Slots are 1024-byte aligned.
//   cp.async: the producer warp's lanes copy 16-byte channel chunks into the
//     no-swizzle layout [CIN/8 chunks][130 pixels][8 channels], keep AHEAD
//     rows in flight and publish the oldest (each lane waits for its own
//     copies, fences them for the tensor core's async proxy and arrives).
//     The host takes it when the input cannot be described by a tensor map.
// RP: row-parallel epilogue.  The eight epilogue warps form two groups of
// four (one per lane quadrant); group g takes the output rows O with O % 2 ==
// g, each thread all COUT channels of its pixel, so two rows' epilogues run
// at once.  Otherwise all eight warps take every row, a warp half of the
// channels.
template <int RING_, int AHEAD_, int NACC_, bool TMA_, bool RP_ = false, int MINB_ = 3>
struct WsCfg {
  static constexpr int RING = RING_, AHEAD = AHEAD_, NACC = NACC_, MINB = MINB_;
  static constexpr bool TMA = TMA_, RP = RP_;
  static constexpr int THREADS = 320;
  static_assert(NACC >= 4, "a row-streaming window holds three slots while one is read");
  static_assert(TMA ? RING >= 2 : RING >= AHEAD + 1, "the ring must hold the rows in flight and the row read");
};

template <int CIN, int COUT, class CFG>
struct SmemWS {
  static constexpr int NC = CIN / 8;
  static constexpr int ROWB = (FTP + 2) * 16;                      // cp.async: bytes of one channel chunk of a row
  static constexpr int SLOT = CFG::TMA ? ((FTP + 2) * CIN * 2 + 1023) / 1024 * 1024 : NC * ROWB;
  static constexpr int WB = 9 * NC * COUT * 16;                    // multiple of 1024
  static constexpr int BIAS = WB + CFG::RING * SLOT;
  static constexpr int BAR = BIAS + 4 * COUT;                      // 8-byte aligned
  static constexpr int NBAR = 2 * CFG::RING + 2 * CFG::NACC + 1;   // full, empty, tfull, tempty, drain
  static constexpr int MISC = BAR + 8 * NBAR;                      // tensor-memory address, abort flag
  static constexpr int BYTES = MISC + 16;
  static constexpr int ALLOC = BYTES + (CFG::TMA ? 1024 : 0);      // room to align the base to 1024 bytes
};

// The input of a launch as a tensor map (TMA producer): dimensions
// {CIN, W, H, N}, box {CIN, 130, 1, 1}.
struct ConvMaps {
  CUtensorMap in;
};

__device__ __forceinline__ void bar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(bar)) : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load4(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                          uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(saddr(bar))
      : "memory");
}

// K-major descriptor of a TMA-staged row (pixels of 2 CIN bytes; 64-byte
// swizzle for CIN 32, 32-byte for CIN 16; 8-row groups 16 CIN bytes apart).
template <int CIN>
__device__ __forceinline__ uint64_t sdesc_sw(uint32_t addr) {
  constexpr uint32_t sbo = 16 * CIN;
  constexpr uint64_t layout = CIN == 32 ? 4 : 6;
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
         ((uint64_t)1 << 46) | (layout << 61);
}

// Bounded wait for the completion of `parity`; false (and the abort flag
// raised) when it runs out or another role has aborted.
__device__ __forceinline__ bool ws_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
  for (int it = 0; it < SPIN_LIMIT; ++it) {
    if (bar_try(bar, parity)) return true;
    if ((it & 1023) == 1023 && *abort_flag) return false;
  }
  if (atomicExch(const_cast<int *>(abort_flag), 1) == 0) atomicAdd(&g_conv_timeouts, 1);
  return false;
}

// Tiles of 128 pixels x th rows, numbered image, row band, column: block b
// takes tiles b, b + G, ..., so the GPU sweeps an image band by band and
// blocks on neighbouring tiles share their halo rows in L2.  Each tile
// streams its th rows plus the two halo rows.
struct WsTile {
  int img, x0, y0, rows;
};
struct WsWalk {
  long long t, ntiles;
  int G, tiles_x, tiles_y, th, H;
  __device__ WsWalk(int b, int G_, int N, int tiles_x_, int H_, int th_) {
    tiles_x = tiles_x_;
    th = th_;
    H = H_;
    tiles_y = (H_ + th_ - 1) / th_;
    ntiles = (long long)N * tiles_x_ * tiles_y;
    t = b;
    G = G_;
  }
  __device__ bool next(WsTile &s) {
    if (t >= ntiles) return false;
    const long long per_img = (long long)tiles_x * tiles_y;
    const long long img = t / per_img, rem = t - img * per_img;
    const int band = (int)(rem / tiles_x), tx = (int)(rem - (long long)band * tiles_x);
    s.img = (int)img;
    s.x0 = tx * FTP;
    s.y0 = band * th;
    s.rows = min(th, H - s.y0);
    t += G;
    return true;
  }
};

template <int CIN, int COUT, int MODE, class CFG>
__global__ void __launch_bounds__(CFG::THREADS, CFG::MINB) k_conv3x3_ws(ConvArgs a, int tiles_x, int th,
                                                             const __grid_constant__ ConvMaps maps) {
  constexpr int RING = CFG::RING, NACC = CFG::NACC, THREADS = CFG::THREADS;
  constexpr int MMA_WARP = 1, EPI0 = 2;
  constexpr int SW = COUT;  // tensor-memory columns per accumulator slot
  constexpr int TALLOC = NACC * SW <= 32 ? 32 : (NACC * SW <= 64 ? 64 : (NACC * SW <= 128 ? 128 : 256));
  using S = SmemWS<CIN, COUT, CFG>;
  static_assert(COUT % 16 == 0 && COUT <= TCOLS && CIN % 16 == 0 && CIN <= 32, "tile shape");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw;
  if constexpr (CFG::TMA) smem += (1024u - (saddr(smem_raw) & 1023u)) & 1023u;
  unsigned char *sw = smem;
  unsigned char *sx = smem + S::WB;
  float *sbias = reinterpret_cast<float *>(smem + S::BIAS);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + S::BAR);
  uint64_t *full = bars, *empty = bars + RING, *tfull = bars + 2 * RING, *tempty = tfull + NACC;
  uint64_t *drain = tempty + NACC;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + S::MISC);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + S::MISC + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t plane = (size_t)a.H * a.W;

  if (tid == 0) {
    for (int k = 0; k < RING; ++k) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(saddr(full + k)), "r"(CFG::TMA ? 1 : 32));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(empty + k)));
    }
    for (int k = 0; k < NACC; ++k) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(tfull + k)));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(saddr(tempty + k)), "r"(CFG::RP ? 128 : 256));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(drain)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *abort_flag = 0;
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                 "r"(TALLOC));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  if (tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.f;
  // weights [dx][k chunk][dy = 2, 1, 0][COUT][8 k values]: the B operand of an
  // input row's (dx, channel step) MMA, up to three output rows stacked
  for (int v = tid; v < 9 * S::NC * COUT; v += THREADS) {
    const int co = v % COUT, d = (v / COUT) % 3, kc = (v / (3 * COUT)) % S::NC, dx = v / (3 * COUT * S::NC);
    const int tap = 3 * (2 - d) + dx;
    cp_async16(sw + (((dx * S::NC + kc) * 3 + d) * COUT + co) * 16, a.w + (size_t)co * 9 * CIN + tap * CIN + kc * 8,
               16);
  }
  cp_async_wait_all();
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t wbase = saddr(sw), xbase = saddr(sx);

  if (warp == 0) {
    if constexpr (CFG::TMA) {
      // ---- producer: one tensor copy per row ----
      if (lane == 0) {
        uint32_t L = 0;  // rows issued
        bool ok = true;
        WsWalk walk(blockIdx.x, gridDim.x, a.N, tiles_x, a.H, th);
        WsTile T;
        while (ok && walk.next(T)) {
          for (int r = 0; r < T.rows + 2; ++r, ++L) {
            const int slot = L % RING;
            const uint32_t use = L / RING;
            if (use > 0 && !ws_wait(empty + slot, (use - 1) & 1u, abort_flag)) {
              ok = false;
              break;
            }
            bar_expect(full + slot, (FTP + 2) * CIN * 2);
            tma_load4(xbase + slot * S::SLOT, &maps.in, 0, T.x0 - 1, T.y0 - 1 + r, T.img, full + slot);
          }
        }
        // every copy issued has landed before the block leaves (bounded; the
        // last use of each slot is the one to wait for)
        for (uint32_t k = L > (uint32_t)RING ? L - RING : 0; k < L; ++k) {
          bool done = false;
          for (int it = 0; it < SPIN_LIMIT && !done; ++it) done = bar_try(full + k % RING, (k / RING) & 1u);
          if (!done) atomicAdd(&g_conv_timeouts, 1);
        }
      }
      __syncwarp();
    } else {
      // ---- producer: lanes copy 16-byte channel chunks ----
      uint32_t L = 0, pub = 0;  // rows issued, rows published
      bool ok = true;
      WsWalk walk(blockIdx.x, gridDim.x, a.N, tiles_x, a.H, th);
      WsTile T;
      while (ok && walk.next(T)) {
        const bf16 *xi = a.x + (size_t)T.img * plane * CIN;
        for (int r = 0; r < T.rows + 2 && ok; ++r, ++L) {
          const int slot = L % RING;
          const uint32_t use = L / RING;
          if (use > 0 && !ws_wait(empty + slot, (use - 1) & 1u, abort_flag)) {
            ok = false;
            break;
          }
          const int yy = T.y0 - 1 + r;
          unsigned char *dst = sx + slot * S::SLOT;
          for (int v = lane; v < (FTP + 2) * S::NC; v += 32) {
            const int col = v / S::NC, c8 = v % S::NC, xx = T.x0 + col - 1;
            const bool in = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
            const bf16 *src = in ? xi + ((size_t)yy * a.W + xx) * CIN + c8 * 8 : xi;
            cp_async16(dst + c8 * S::ROWB + col * 16, src, in ? 16 : 0);
          }
          cp_async_commit();
          if (L + 1 - pub > (uint32_t)CFG::AHEAD) {  // publish the oldest row in flight
            asm volatile("cp.async.wait_group %0;\n" ::"n"(CFG::AHEAD) : "memory");
            fence_async_smem();
            bar_arrive(full + pub % RING);
            ++pub;
          }
        }
      }
      cp_async_wait_all();
      fence_async_smem();
      for (; pub < L; ++pub) bar_arrive(full + pub % RING);
    }
  } else if (warp == MMA_WARP) {
    // ---- MMA issuer ----
    if (lane == 0) {
      // one pass per staged input row t of a tile (image row y0 - 1 + t): it
      // feeds output rows t - 2 (dy = 2), t - 1 (dy = 1) and t (dy = 0) of the
      // tile, whose accumulators sit in consecutive slots; out(t) starts here
      // (its first MMA does not accumulate) and out(t - 2) is complete after
      uint32_t L = 0, O = 0;  // input rows and output rows of the tiles so far
      bool ok = true;
      auto run = [&](uint32_t Ob, int t, int oa, int ob, uint64_t ad, uint32_t bchunk, uint32_t acc) {
        // outputs oa..ob (consecutive slots, split where the slot ring wraps)
        const int sa = (int)((Ob + oa) % NACC);
        const int cnt = ob - oa + 1, c1 = sa + cnt <= NACC ? cnt : NACC - sa;
        const int d0 = oa - (t - 2);  // B block of output oa: dy = 2 - d0
        mma(tmem + sa * SW, ad, sdesc(bchunk + d0 * COUT * 16, 3 * COUT * 16, 128), idesc(128, c1 * COUT), acc);
        if (c1 < cnt)
          mma(tmem, ad, sdesc(bchunk + (d0 + c1) * COUT * 16, 3 * COUT * 16, 128), idesc(128, (cnt - c1) * COUT), acc);
      };
      WsWalk walk(blockIdx.x, gridDim.x, a.N, tiles_x, a.H, th);
      WsTile T;
      while (ok && walk.next(T)) {
        for (int t = 0; t < T.rows + 2; ++t) {
          const uint32_t Lt = L + t;
          if (!ws_wait(full + Lt % RING, (Lt / RING) & 1u, abort_flag)) {
            ok = false;
            break;
          }
          const int o1 = t - 2 > 0 ? t - 2 : 0, o2 = t < T.rows - 1 ? t : T.rows - 1;
          const bool fresh = t <= T.rows - 1;
          if (fresh) {
            const uint32_t Og = O + t, use = Og / NACC;
            if (use > 0 && !ws_wait(tempty + Og % NACC, (use - 1) & 1u, abort_flag)) {
              ok = false;
              break;
            }
          }
          fence_after();
          const uint32_t rbase = xbase + (Lt % RING) * S::SLOT;
#pragma unroll
          for (int dx = 0; dx < 3; ++dx) {
#pragma unroll
            for (int cc = 0; cc < CIN; cc += 16) {
              const uint64_t ad = CFG::TMA ? sdesc_sw<CIN>(rbase + dx * CIN * 2 + cc * 2)
                                           : sdesc(rbase + (cc / 8) * S::ROWB + dx * 16, S::ROWB, 128);
              const uint32_t bchunk = wbase + (dx * S::NC + cc / 8) * 3 * COUT * 16;
              if (dx == 0 && cc == 0 && fresh) {
                if (t - 1 >= o1) run(O, t, o1, t - 1, ad, bchunk, 1u);
                run(O, t, t, t, ad, bchunk, 0u);
              } else {
                run(O, t, o1, o2, ad, bchunk, 1u);
              }
            }
          }
          commit(empty + Lt % RING);  // the input row has fed every output row it feeds
          if (t >= 2) commit(tfull + (O + t - 2) % NACC);
        }
        L += T.rows + 2;
        O += T.rows;
      }
      // every MMA issued has completed before the block leaves (bounded, and
      // waited for even after an abort: tensor memory is freed below)
      commit(drain);
      bool drained = false;
      for (int it = 0; it < SPIN_LIMIT && !drained; ++it) drained = bar_try(drain, 0u);
      if (!drained) atomicAdd(&g_conv_timeouts, 1);
    }
    __syncwarp();
  } else {
    // ---- epilogue ----
    constexpr bool RP = CFG::RP;
    constexpr int CW = RP ? COUT : COUT / 2;  // channels per thread
    const int ew = warp - EPI0, quad = warp & 3, grp = ew >> 2, half = RP ? 0 : grp;
    uint32_t O = 0;
    bool ok = true;
    WsWalk walk(blockIdx.x, gridDim.x, a.N, tiles_x, a.H, th);
    WsTile T;
    while (ok && walk.next(T)) {
      const int xx = T.x0 + 32 * quad + lane;
      for (int i = 0; i < T.rows; ++i, ++O) {
        if (RP && (int)(O & 1u) != grp) continue;
        const int y = T.y0 + i;
        uint4 gzv[MODE == 2 ? CW / 8 : 1];
        if (MODE == 2 && xx < a.W) {
          const uint4 *gp = reinterpret_cast<const uint4 *>(
              a.gz + ((size_t)T.img * plane + (size_t)y * a.W + xx) * COUT + half * CW);
#pragma unroll
          for (int q = 0; q < (MODE == 2 ? CW / 8 : 1); ++q) gzv[q] = gp[q];
        }
        const int acc_i = O % NACC;
        if (!ws_wait(tfull + acc_i, (O / NACC) & 1u, abort_flag)) {
          ok = false;
          break;
        }
        fence_after();
        float acc[CW];
        {
          const uint32_t ta = tmem + ((uint32_t)(32 * quad) << 16) + acc_i * SW + half * CW;
          if constexpr (CW >= 16) {
#pragma unroll
            for (int c0 = 0; c0 < CW; c0 += 16) {
              float v[16];
              tld16(ta + c0, v);
#pragma unroll
              for (int k = 0; k < 16; ++k) acc[c0 + k] = v[k];
            }
          } else {
            float v[8];
            tld8(ta, v);
#pragma unroll
            for (int k = 0; k < CW; ++k) acc[k] = v[k];
          }
        }
        fence_before();
        bar_arrive(tempty + acc_i);
        if (xx < a.W) {
          const size_t pix = (size_t)T.img * plane + (size_t)y * a.W + xx;
#pragma unroll
          for (int c = 0; c < CW; ++c) acc[c] += sbias[half * CW + c];
          if (a.out32 && half == 0) a.out32[pix] = acc[0];
          uint4 zo[CW / 8], oo[CW / 8];
#pragma unroll
          for (int q = 0; q < CW / 8; ++q) {
            __nv_bfloat162 *zp = reinterpret_cast<__nv_bfloat162 *>(&zo[q]);
            __nv_bfloat162 *op = reinterpret_cast<__nv_bfloat162 *>(&oo[q]);
            const __nv_bfloat162 *gq = reinterpret_cast<const __nv_bfloat162 *>(&gzv[MODE == 2 ? q : 0]);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              const float z0 = acc[8 * q + 2 * h], z1 = acc[8 * q + 2 * h + 1];
              float o0 = z0, o1 = z1;
              if (MODE == 1) {
                zp[h] = __floats2bfloat162_rn(z0, z1);
                o0 = gelu_hw(z0);
                o1 = gelu_hw(z1);
              } else if (MODE == 2) {
                o0 = z0 * gelu_grad_hw(__low2float(gq[h]));
                o1 = z1 * gelu_grad_hw(__high2float(gq[h]));
              }
              op[h] = __floats2bfloat162_rn(o0, o1);
            }
          }
          if (MODE == 1 && a.z) {
            uint4 *zd = reinterpret_cast<uint4 *>(a.z + pix * COUT + half * CW);
#pragma unroll
            for (int q = 0; q < CW / 8; ++q) zd[q] = zo[q];
          }
          if (a.out) {
            uint4 *od = reinterpret_cast<uint4 *>(a.out + pix * COUT + half * CW);
#pragma unroll
            for (int q = 0; q < CW / 8; ++q) od[q] = oo[q];
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == MMA_WARP)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TALLOC));
}

}  // namespace tc

// Weight and bias gradients: dW[co][tap][ci] = sum_p dz[p][co] x[p + off(tap)][ci]
// as a GEMM with M = COUT, N = 9*CIN, K = pixels; db[co] = sum_p dz[p][co].
// Block b walks row segments b, b + G, ...; A (dz, stored [p][co]) and B (the
// shifted input, stored [p][ci]) fragments come from ldmatrix.trans.  Each
// block writes its partial sums; k_sum_partials adds them in block order.
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv_dw(const bf16 *__restrict__ x, const bf16 *__restrict__ dz,
                                                 float *__restrict__ part, int N, int H, int W) {
  constexpr int PS = CIN + 8, ZS = COUT + 8;
  constexpr int MT = COUT / 16;
  constexpr int NTT = 9 * CIN / 8;
  constexpr int NPW = (NTT + 3) / 4;
  constexpr int NW = COUT * 9 * CIN + COUT;
  constexpr int VX = CIN / 8, VZ = COUT / 8;
  __shared__ __align__(16) bf16 sx[3][TP + 2][PS];
  __shared__ __align__(16) bf16 sz[TP][ZS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const size_t plane = (size_t)H * W;
  const int segs = (W + TP - 1) / TP;
  const long long tiles = (long long)N * H * segs;
  float acc[MT][NPW][4];
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int q = 0; q < NPW; ++q) acc[m][q][0] = acc[m][q][1] = acc[m][q][2] = acc[m][q][3] = 0.f;
  float bacc = 0.f;
  for (long long tt = blockIdx.x; tt < tiles; tt += gridDim.x) {
    const int seg = (int)(tt % segs);
    const long long rr = tt / segs;
    const int y = (int)(rr % H), img = (int)(rr / H), x0 = seg * TP;
    __syncthreads();
    for (int v = tid; v < 3 * (TP + 2) * VX; v += 128) {
      const int c8 = v % VX, col = (v / VX) % (TP + 2), r = v / (VX * (TP + 2));
      const int yy = y + r - 1, xx = x0 + col - 1;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (yy >= 0 && yy < H && xx >= 0 && xx < W)
        val = *reinterpret_cast<const uint4 *>(x + ((size_t)img * plane + (size_t)yy * W + xx) * CIN + c8 * 8);
      *reinterpret_cast<uint4 *>(&sx[r][col][c8 * 8]) = val;
    }
    for (int v = tid; v < TP * VZ; v += 128) {
      const int c8 = v % VZ, p = v / VZ, xx = x0 + p;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (xx < W) val = *reinterpret_cast<const uint4 *>(dz + ((size_t)img * plane + (size_t)y * W + xx) * COUT + c8 * 8);
      *reinterpret_cast<uint4 *>(&sz[p][c8 * 8]) = val;
    }
    __syncthreads();
    if (tid < COUT)
      for (int p = 0; p < TP; ++p) bacc += __bfloat162float(sz[p][tid]);
#pragma unroll
    for (int ks = 0; ks < TP / 16; ++ks) {
      const int p0 = ks * 16;
      uint32_t af[MT][4];
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        const int j = lane >> 3, r = lane & 7;
        ldsm_x4_trans(af[m], &sz[p0 + (j >> 1) * 8 + r][m * 16 + (j & 1) * 8]);
      }
#pragma unroll
      for (int q = 0; q < NPW; ++q) {
        const int nt = warp + 4 * q;
        if (nt < NTT) {
          const int n0 = nt * 8, tap = n0 / CIN, ci0 = n0 % CIN, dy = tap / 3, dx = tap % 3;
          const int j = (lane >> 3) & 1, r = lane & 7;
          uint32_t bfr[2];
          ldsm_x2_trans(bfr, &sx[dy][p0 + j * 8 + r + dx][ci0]);
#pragma unroll
          for (int m = 0; m < MT; ++m) mma_bf16(acc[m][q], af[m], bfr);
        }
      }
    }
  }
  float *out = part + (size_t)blockIdx.x * NW;
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int q = 0; q < NPW; ++q) {
      const int nt = warp + 4 * q;
      if (nt < NTT) {
        const int nn = nt * 8 + 2 * t, ca = m * 16 + g, cb = ca + 8;
        out[(size_t)ca * 9 * CIN + nn] = acc[m][q][0];
        out[(size_t)ca * 9 * CIN + nn + 1] = acc[m][q][1];
        out[(size_t)cb * 9 * CIN + nn] = acc[m][q][2];
        out[(size_t)cb * 9 * CIN + nn + 1] = acc[m][q][3];
      }
    }
  if (tid < COUT) out[COUT * 9 * CIN + tid] = bacc;
}

__global__ void k_sum_partials(const float *part, int nparts, int n, float *out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nparts; ++b) s += part[(size_t)b * n + k];
    out[k] = s;
  }
}

// Wt[ci][tap][co] = W[co][8 - tap][ci]: the weights of the input-gradient convolution.
__global__ void k_flip(const bf16 *w, bf16 *wt, int cin, int cout) {
  const int n = cin * 9 * cout;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int co = k % cout, tap = (k / cout) % 9, ci = k / (9 * cout);
    wt[k] = w[((size_t)co * 9 + (8 - tap)) * cin + ci];
  }
}

// Adam on FP32 master weights (gradient clipped elementwise); refreshes the
// BF16 copy the convolutions read.
__global__ void k_adam(float *wt, float *m, float *v, const float *grad, bf16 *wbf, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2, float clip, float gscale) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    float gk = grad[k] * gscale;
    gk = fminf(fmaxf(gk, -clip), clip);
    m[k] = b1 * m[k] + (1.f - b1) * gk;
    v[k] = b2 * v[k] + (1.f - b2) * gk * gk;
    const float mh = m[k] / c1, vh = v[k] / c2;
    wt[k] -= lr * mh / (sqrtf(vh) + eps);
    if (wbf) wbf[k] = __float2bfloat16(wt[k]);
  }
}

// Network input of crop b at (y, x): u / su, log(rx / rho) / 4, (u - uprev) / sd,
// then 13 zero channels.  Cells outside the domain give zeros.
__global__ void k_features(const tl_warm_crop *crops, int B, int H, int W, bf16 *feat) {
  const long long n = (long long)B * H * W;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(k % W), y = (int)((k / W) % H), b = (int)(k / ((long long)H * W));
    const tl_warm_crop cr = crops[b];
    const int gx = cr.ox + x, gy = cr.oy + y;
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
    if (gx >= 0 && gx < cr.nx && gy >= 0 && gy < cr.ny) {
      const size_t c = (size_t)gy * cr.pitch + gx;
      const double u = cr.u[c];
      f0 = (float)(u * cr.inv_su);
      f1 = 0.25f * (float)log(cr.rx / cr.rho[c]);
      f2 = (float)((u - cr.uprev[c]) * cr.inv_sd);
    }
    __nv_bfloat162 p0 = __floats2bfloat162_rn(f0, f1), p1 = __floats2bfloat162_rn(f2, 0.f);
    uint4 v0 = make_uint4(*reinterpret_cast<uint32_t *>(&p0), *reinterpret_cast<uint32_t *>(&p1), 0, 0);
    uint4 *dst = reinterpret_cast<uint4 *>(feat + k * 16);
    dst[0] = v0;
    dst[1] = make_uint4(0, 0, 0, 0);
  }
}

// Face coefficient between two cells of the crop's domain (0 across the domain
// boundary: the reflective halo carries no flux).
__device__ __forceinline__ double face_k(const tl_warm_crop &cr, double r, int ax, int ay, int bx, int by) {
  if (ax < 0 || ay < 0 || bx >= cr.nx || by >= cr.ny) return 0.0;
  const double ra = cr.rho[(size_t)ay * cr.pitch + ax], rb = cr.rho[(size_t)by * cr.pitch + bx];
  return r * (ra + rb) / (2.0 * ra * rb);
}

// (A v)(gx, gy) = v + sum over faces k (v - v_nbr) for a field v given on crop
// coordinates through `at(x, y)`.
template <class F>
__device__ __forceinline__ double apply_a(const tl_warm_crop &cr, int x, int y, F at) {
  const int gx = cr.ox + x, gy = cr.oy + y;
  const double v = at(x, y);
  double s = v;
  s += face_k(cr, cr.rx, gx - 1, gy, gx, gy) * (v - at(x - 1, y));
  s += face_k(cr, cr.rx, gx, gy, gx + 1, gy) * (v - at(x + 1, y));
  s += face_k(cr, cr.ry, gx, gy - 1, gx, gy) * (v - at(x, y - 1));
  s += face_k(cr, cr.ry, gx, gy, gx, gy + 1) * (v - at(x, y + 1));
  return s;
}

// Loss pass 1: r = d - A((1 + g) d) on the crop's loss region
// [m, W - m) x [m, H - m) with d = u - uprev, in units of the deck's rms
// increment (s = inv_sd); partial sums of (s r)^2 and (s d)^2 per block and crop.
__global__ void __launch_bounds__(256) k_loss_resid(const tl_warm_crop *crops, int H, int W, int margin,
                                                    const float *g, double *resid, double *sums) {
  const int b = blockIdx.y;
  const tl_warm_crop cr = crops[b];
  const float *gb = g + (size_t)b * H * W;
  double *rb = resid + (size_t)b * H * W;
  auto d_at = [&](int x, int y) {
    const size_t c = (size_t)(cr.oy + y) * cr.pitch + (cr.ox + x);
    return cr.u[c] - cr.uprev[c];
  };
  auto x_at = [&](int x, int y) { return (1.0 + (double)gb[(size_t)y * W + x]) * d_at(x, y); };
  const int LW = W - 2 * margin, LH = H - 2 * margin;
  double srr = 0.0, sdd = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < LW * LH; k += gridDim.x * blockDim.x) {
    const int x = margin + k % LW, y = margin + k / LW;
    const double d = d_at(x, y);
    const double r = d - apply_a(cr, x, y, x_at);
    rb[(size_t)y * W + x] = r;
    const double rs = r * cr.inv_sd, ds = d * cr.inv_sd;
    srr += rs * rs;
    sdd += ds * ds;
  }
  __shared__ double s1[256], s2[256];
  s1[threadIdx.x] = srr;
  s2[threadIdx.x] = sdd;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    sums[((size_t)b * gridDim.x + blockIdx.x) * 2] = s1[0];
    sums[((size_t)b * gridDim.x + blockIdx.x) * 2 + 1] = s2[0];
  }
}

// Loss pass 2 (one thread per crop): crop_loss[2b] = mean (s r)^2 over the loss
// region, crop_loss[2b+1] = mean (s d)^2 (the plain start's value).
__global__ void k_loss_fold(const double *sums, int B, int nblk, double ncells, double *crop_loss) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  double rr = 0.0, dd = 0.0;
  for (int k = 0; k < nblk; ++k) {
    rr += sums[((size_t)b * nblk + k) * 2];
    dd += sums[((size_t)b * nblk + k) * 2 + 1];
  }
  crop_loss[2 * b] = rr / ncells;
  crop_loss[2 * b + 1] = dd / ncells;
}

// Loss pass 3: for L = mean over crops of crop_loss[2b] (objective 0) or of
// log(crop_loss[2b] / crop_loss[2b+1]) (objective 1),
// dL/dg = -2 s^2 (A r~) d / (ncells B) [/ crop_loss[2b]] one cell beyond the
// loss region (r~ = r on the loss region, 0 elsewhere), written as channel 0
// of the output gradient; every other channel and cell gets 0.
__global__ void k_loss_grad(const tl_warm_crop *crops, int B, int H, int W, int margin, const double *resid,
                            double ncells, const double *crop_loss, int objective, bf16 *dz) {
  const long long n = (long long)B * H * W;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(k % W), y = (int)((k / W) % H), b = (int)(k / ((long long)H * W));
    float gv = 0.f;
    if (x >= margin - 1 && x < W - margin + 1 && y >= margin - 1 && y < H - margin + 1) {
      const tl_warm_crop cr = crops[b];
      const double *rb = resid + (size_t)b * H * W;
      auto r_at = [&](int xx, int yy) {
        return (xx >= margin && xx < W - margin && yy >= margin && yy < H - margin) ? rb[(size_t)yy * W + xx] : 0.0;
      };
      const double ar = apply_a(cr, x, y, r_at);
      const size_t c = (size_t)(cr.oy + y) * cr.pitch + (cr.ox + x);
      const double d = cr.u[c] - cr.uprev[c];
      double scale = -2.0 * cr.inv_sd * cr.inv_sd / (ncells * B);
      if (objective == 1) scale = crop_loss[2 * b] > 0 ? scale / crop_loss[2 * b] : 0.0;
      gv = (float)(ar * d * scale);
    }
    __nv_bfloat162 p0 = __floats2bfloat162_rn(gv, 0.f);
    uint4 *dst = reinterpret_cast<uint4 *>(dz + k * 16);
    dst[0] = make_uint4(*reinterpret_cast<uint32_t *>(&p0), 0, 0, 0);
    dst[1] = make_uint4(0, 0, 0, 0);
  }
}

inline int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 16) b = 152LL * 16;
  return (int)(b < 1 ? 1 : b);
}

// The forward kernel: the warp-specialised tcgen05 kernel by default;
// TEALEAF_GB300_CONV=tc selects the row-synchronous tcgen05 kernel and
// TEALEAF_GB300_CONV=mma the warp-level mma.sync one (both kept for comparison).
int conv_kind() {
  static const int v = [] {
    const char *e = getenv("TEALEAF_GB300_CONV");
    if (e && !strcmp(e, "mma")) return 2;
    if (e && !strcmp(e, "tc")) return 1;
    return 0;
  }();
  return v;
}
bool conv_use_mma() { return conv_kind() == 2; }

int conv_sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        n < 1)
      n = 152;
  }
  return n;
}

// The warp-specialised kernel's producer and epilogue (TEALEAF_GB300_CONV_WS):
//   0 (default) a tensor copy per row into a 4-slot ring; the GELU forward
//     (mode 1) with the row-parallel epilogue at three blocks per SM, the
//     plain output (0) and the input gradient (2) with every epilogue warp
//     on every row at four blocks per SM (each measured best for its mode);
//   1 a tensor copy per row, every epilogue warp on every row (half the
//     channels), three blocks per SM, every mode;
//   2 cp.async channel chunks into a 6-slot ring with 3 rows ahead, every
//     epilogue warp on every row (also taken when the input admits no
//     tensor map).
// All keep 4 accumulator slots.
int conv_ws_cfg() {
  static const int v = [] {
    const char *e = getenv("TEALEAF_GB300_CONV_WS");
    const int k = e ? atoi(e) : 0;
    return (k >= 0 && k <= 2) ? k : 0;
  }();
  return v;
}

// cuTensorMapEncodeTiled from the driver, looked up once.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// The input as a 4-D tensor map {CIN, W, H, N} (pixel strides 2 CIN bytes)
// with box {CIN, FTP + 2, 1, 1}, zero fill outside, the 64-byte (CIN 32) or
// 32-byte (CIN 16) swizzle; false when it cannot be made.
template <int CIN>
bool input_map(const ConvArgs &a, CUtensorMap *m) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(a.x) & 15u) != 0) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)CIN, (cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.N};
  const cuuint64_t strides[3] = {(cuuint64_t)CIN * 2, (cuuint64_t)a.W * CIN * 2, (cuuint64_t)a.H * a.W * CIN * 2};
  const cuuint32_t box[4] = {(cuuint32_t)CIN, (cuuint32_t)(FTP + 2), 1, 1}, es[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(a.x), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CIN == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// A persistent grid: as many blocks as fit on the GPU at once (by shared
// memory and tensor memory, at most MAXB per SM), at most one per tile.
template <int CIN, int COUT, int MODE, class CFG, int MAXB>
void launch_ws(const ConvArgs &a, const tc::ConvMaps &maps, cudaStream_t st) {
  constexpr int smem = tc::SmemWS<CIN, COUT, CFG>::ALLOC;
  // blocks per SM: what fits in the 228 KB of shared memory (1 KB reserved
  // per block) and in the 512 tensor-memory columns
  constexpr int cols = CFG::NACC * COUT;
  constexpr int talloc = cols <= 32 ? 32 : (cols <= 64 ? 64 : (cols <= 128 ? 128 : 256));
  constexpr int fit = 233472 / (smem + 1024), tfit = 512 / talloc;
  constexpr int per_sm0 = fit < tfit ? fit : tfit;
  constexpr int per_sm = per_sm0 < 1 ? 1 : (per_sm0 > MAXB ? MAXB : per_sm0);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(tc::k_conv3x3_ws<CIN, COUT, MODE, CFG>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(tc::k_conv3x3_ws<CIN, COUT, MODE, CFG>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    attr = true;
  }
  const int tiles_x = (a.W + FTP - 1) / FTP;
  const long long cap = (long long)per_sm * conv_sm_count();
  // tile height: 16 rows when that gives every block slot a tile (measured
  // best: a short last wave costs less than the halo rows of shorter tiles,
  // the blocks left on an SM taking its whole bandwidth); on smaller images
  // the height whose last block finishes first, counting each tile's rows
  // plus its two halo rows (ties to the taller tile); or the height
  // TEALEAF_GB300_CONV_ROWS names (1..16)
  static const int rows_env = [] {
    const char *e = getenv("TEALEAF_GB300_CONV_ROWS");
    const int k = e ? atoi(e) : 0;
    return (k >= 1 && k <= 16) ? k : 0;
  }();
  int th = 16;
  long long best = -1, blocks = 1;
  const bool full = (long long)a.N * tiles_x * ((a.H + 15) / 16) >= cap;
  for (int h = 16; h >= 1; --h) {
    if (rows_env ? h != rows_env : (full && h != 16)) continue;
    const long long tiles = (long long)a.N * tiles_x * ((a.H + h - 1) / h);
    const long long g = tiles < cap ? tiles : cap;
    const long long cost = (tiles + g - 1) / g * (h + 2);
    if (best < 0 || cost < best) {
      best = cost;
      th = h;
      blocks = g;
    }
  }
  tc::k_conv3x3_ws<CIN, COUT, MODE, CFG><<<(int)blocks, CFG::THREADS, smem, st>>>(a, tiles_x, th, maps);
}

template <int CIN, int COUT, int MODE>
void launch_conv_mode(const ConvArgs &a, cudaStream_t st) {
  const dim3 grid((a.W + FTP - 1) / FTP, (a.H + FRB - 1) / FRB, a.N);
  if (conv_use_mma()) {
    constexpr int smem = conv_smem_bytes<CIN, COUT>();
    static bool attr = false;  // the dynamic shared memory limit, set once per kernel
    if (!attr) {
      cudaFuncSetAttribute(k_conv3x3<CIN, COUT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      attr = true;
    }
    k_conv3x3<CIN, COUT, MODE><<<grid, 128, smem, st>>>(a);
    return;
  }
  if (conv_kind() == 1) {
    constexpr int smem = tc::Smem<CIN, COUT>::BYTES;
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(tc::k_conv3x3_tc<CIN, COUT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      attr = true;
    }
    tc::k_conv3x3_tc<CIN, COUT, MODE><<<grid, 256, smem, st>>>(a);
    return;
  }
  // GELU forward: the row-parallel epilogue at three blocks per SM; plain
  // output and input gradient: every epilogue warp on every row at four
  // blocks per SM (registers capped at 48; measured faster for those two)
  using TmaCfg = tc::WsCfg<4, 1, 4, true, MODE == 1, MODE == 1 ? 3 : 4>;
  constexpr int TMA_MAXB = MODE == 1 ? 3 : 4;
  using TmaCfgAll = tc::WsCfg<4, 1, 4, true, false>;
  using CpCfg = tc::WsCfg<6, 3, 4, false>;
  tc::ConvMaps maps;
  memset(&maps, 0, sizeof(maps));
  const int cfg = conv_ws_cfg();
  if (cfg != 2 && input_map<CIN>(a, &maps.in)) {
    if (cfg == 1) launch_ws<CIN, COUT, MODE, TmaCfgAll, 3>(a, maps, st);
    else launch_ws<CIN, COUT, MODE, TmaCfg, TMA_MAXB>(a, maps, st);
  } else {
    launch_ws<CIN, COUT, MODE, CpCfg, 3>(a, maps, st);
  }
}

template <int CIN, int COUT>
void launch_conv(const ConvArgs &a, int mode, cudaStream_t st) {
  if (mode == 0) launch_conv_mode<CIN, COUT, 0>(a, st);
  else if (mode == 1) launch_conv_mode<CIN, COUT, 1>(a, st);
  else launch_conv_mode<CIN, COUT, 2>(a, st);
}

}  // namespace

int tl_conv_forward(const void *x, const void *w, const float *bias, const void *gz, void *z, void *out, float *out32,
                    int N, int H, int W, int cin, int cout, int mode, cudaStream_t st) {
  if (!x || !w || (!out && !out32) || N < 1 || H < 1 || W < 1 || mode < 0 || mode > 2) return TL_ERR_ARG;
  if (mode == 2 && !gz) return TL_ERR_ARG;
  // the kernels move activations and weights in 16-byte vectors
  auto misaligned = [](const void *q, uintptr_t m) { return (reinterpret_cast<uintptr_t>(q) & m) != 0; };
  if (misaligned(x, 15) || misaligned(w, 15) || misaligned(gz, 15) || misaligned(z, 15) || misaligned(out, 15) ||
      misaligned(out32, 3))
    return TL_ERR_ARG;
  if (N > 65535 || (H + FRB - 1) / FRB > 65535) return TL_ERR_ARG;
  if ((long long)N * ((W + FTP - 1) / FTP) * H > (1LL << 40)) return TL_ERR_ARG;
  ConvArgs a;
  a.x = static_cast<const bf16 *>(x);
  a.w = static_cast<const bf16 *>(w);
  a.gz = static_cast<const bf16 *>(gz);
  a.bias = bias;
  a.z = static_cast<bf16 *>(z);
  a.out = static_cast<bf16 *>(out);
  a.out32 = out32;
  a.N = N;
  a.H = H;
  a.W = W;
  if (cin == 16 && cout == 32) launch_conv<16, 32>(a, mode, st);
  else if (cin == 32 && cout == 32) launch_conv<32, 32>(a, mode, st);
  else if (cin == 32 && cout == 16) launch_conv<32, 16>(a, mode, st);
  else return TL_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? TL_OK : TL_ERR_CUDA;
}

extern "C" int tl_conv3x3_forward(const void *x, const void *w, const float *bias, const void *gz, void *z, void *out,
                                  float *out32, int N, int H, int W, int cin, int cout, int mode, void *stream) {
  return tl_conv_forward(x, w, bias, gz, z, out, out32, N, H, W, cin, cout, mode, static_cast<cudaStream_t>(stream));
}

extern "C" int tl_conv_status(int *timeouts) {
  if (!timeouts) return TL_ERR_ARG;
  if (cudaDeviceSynchronize() != cudaSuccess) return TL_ERR_CUDA;
  const int zero = 0;
  if (cudaMemcpyFromSymbol(timeouts, tc::g_conv_timeouts, sizeof(int)) != cudaSuccess ||
      cudaMemcpyToSymbol(tc::g_conv_timeouts, &zero, sizeof(int)) != cudaSuccess)
    return TL_ERR_CUDA;
  return TL_OK;
}

extern "C" int tl_conv3x3_weight_grad(const void *x, const void *dz, float *partials, int nparts, float *dw, int N,
                                      int H, int W, int cin, int cout, void *stream) {
  if (!x || !dz || !partials || !dw || nparts < 1 || N < 1 || H < 1 || W < 1) return TL_ERR_ARG;
  // activations are read in 16-byte vectors, partials and gradients as floats
  if ((reinterpret_cast<uintptr_t>(x) & 15u) || (reinterpret_cast<uintptr_t>(dz) & 15u) ||
      (reinterpret_cast<uintptr_t>(partials) & 3u) || (reinterpret_cast<uintptr_t>(dw) & 3u))
    return TL_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto X = static_cast<const bf16 *>(x);
  auto Z = static_cast<const bf16 *>(dz);
  const int nw = cout * 9 * cin + cout;
  if (cin == 16 && cout == 32) k_conv_dw<16, 32><<<nparts, 128, 0, st>>>(X, Z, partials, N, H, W);
  else if (cin == 32 && cout == 32) k_conv_dw<32, 32><<<nparts, 128, 0, st>>>(X, Z, partials, N, H, W);
  else if (cin == 32 && cout == 16) k_conv_dw<32, 16><<<nparts, 128, 0, st>>>(X, Z, partials, N, H, W);
  else return TL_ERR_ARG;
  k_sum_partials<<<grid_for(nw), 256, 0, st>>>(partials, nparts, nw, dw);
  return cudaGetLastError() == cudaSuccess ? TL_OK : TL_ERR_CUDA;
}

extern "C" int tl_conv3x3_flip(const void *w, void *wt, int cin, int cout, void *stream) {
  if (!w || !wt || cin < 1 || cout < 1) return TL_ERR_ARG;
  k_flip<<<grid_for((long long)cin * 9 * cout), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16 *>(w), static_cast<bf16 *>(wt), cin, cout);
  return cudaGetLastError() == cudaSuccess ? TL_OK : TL_ERR_CUDA;
}

extern "C" int tl_adam_step(float *w, float *m, float *v, const float *grad, void *wbf16, int n, float lr, float b1,
                            float b2, float eps, int step, float clip, float gscale, void *stream) {
  if (!w || !m || !v || !grad || n < 1 || step < 1) return TL_ERR_ARG;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(w, m, v, grad, static_cast<bf16 *>(wbf16), n,
                                                                      lr, b1, b2, eps, c1, c2, clip, gscale);
  return cudaGetLastError() == cudaSuccess ? TL_OK : TL_ERR_CUDA;
}

int tl_warm_features_launch(const tl_warm_crop *crops, int B, int H, int W, void *feat, cudaStream_t st) {
  k_features<<<grid_for((long long)B * H * W), 256, 0, st>>>(crops, B, H, W, static_cast<bf16 *>(feat));
  return cudaGetLastError() == cudaSuccess ? TL_OK : TL_ERR_CUDA;
}

extern "C" int tl_warm_features(const tl_warm_crop *crops, int B, int H, int W, void *feat, void *stream) {
  if (!crops || !feat || B < 1 || H < 1 || W < 1) return TL_ERR_ARG;
  return tl_warm_features_launch(crops, B, H, W, feat, static_cast<cudaStream_t>(stream));
}

extern "C" int tl_warm_loss(const tl_warm_crop *crops, int B, int H, int W, int margin, int objective, const float *g,
                            double *resid, double *sums, int nblk, double *crop_loss, void *dz, void *stream) {
  if (!crops || !g || !resid || !sums || !crop_loss || !dz || B < 1 || B > 65535 || nblk < 1 || margin < 2 ||
      W <= 2 * margin || H <= 2 * margin)
    return TL_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_loss_resid<<<dim3(nblk, B), 256, 0, st>>>(crops, H, W, margin, g, resid, sums);
  const double ncells = (double)(W - 2 * margin) * (H - 2 * margin);
  k_loss_fold<<<(B + 127) / 128, 128, 0, st>>>(sums, B, nblk, ncells, crop_loss);
  k_loss_grad<<<grid_for((long long)B * H * W), 256, 0, st>>>(crops, B, H, W, margin, resid, ncells, crop_loss,
                                                               objective,
                                                               static_cast<bf16 *>(dz));
  return cudaGetLastError() == cudaSuccess ? TL_OK : TL_ERR_CUDA;
}
