// scf_unet_tc.cu -- 3x3 convolutions of the learned preconditioner on the
// fifth-generation tensor cores (tcgen05.mma, accumulators in tensor memory).
//
// Implicit GEMM per tile: D[128 pixels][COUT] = sum over the 9 taps of
// A_tap[128 pixels][CIN] x B_tap[CIN][COUT], BF16 operands from shared
// memory, FP32 accumulation in TMEM (128 lanes = pixels, COUT columns).
//
// Tiles are 128 consecutive pixels of one image row.  A CTA owns a strip of
// rows of one 128-pixel column segment and walks down it, so each tile stages
// only ONE new input row: a ring of four staged rows holds the rows y-1, y,
// y+1 of the current tile and the row y+2 that is loaded while the tensor
// core works on the current tile.  A staged row keeps the 130 pixels
// x0-1 .. x0+128 in the no-swizzle K-major canonical layout (8-pixel x 16-byte
// core matrices, pixels 16 bytes apart inside a channel group, the 8-channel
// groups LBO bytes apart), so the operand of tap (dy, dx) is the staged row
// of y+dy-1 with its start address moved by dx pixels (16 bytes): the
// one-pixel shifts of the 3x3 stencil cost no copies.  The weights of all
// nine taps stay in shared memory in the same layout (8 output channels x
// 16 bytes per core matrix).  Zero padding, nearest upsampling of a
// half-resolution input and the ReLU mask of the backward pass are applied
// while a row is staged.
//
// One thread issues the MMAs of a tile (9 taps x CIN/16 K-steps of
// M=128, N=COUT, K=16) and commits them to an mbarrier; all 128 threads stage
// the next row meanwhile, then wait (bounded) for the commit, read their
// pixel's accumulator row from TMEM (thread t = lane t), add bias / skip,
// apply ReLU and store BF16.  A wait that runs out sets *err, waits once
// more (bounded) for the MMAs in flight, frees the tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>

#include "scf_unet.cuh"

namespace scf {
extern thread_local long long g_launches;  // defined with the multigrid launchers
}  // namespace scf

namespace scf {
namespace {

using bf16 = __nv_bfloat16;
using bf162 = __nv_bfloat162;

constexpr int kTile = 128;      // output pixels per tile = MMA M = threads per CTA
constexpr int kRing = 4;        // staged rows
constexpr int kSpins = 1 << 20; // bounded mbarrier polls (each suspends at most ~1 us)
constexpr unsigned kPollNs = 1024;

__device__ __forceinline__ unsigned saddr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// --- tcgen05 / mbarrier primitives -----------------------------------------
__device__ __forceinline__ void bar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool bar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(parity), "n"(kPollNs)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool bar_wait_bounded(uint64_t* bar, unsigned parity) {
  for (int i = 0; i < kSpins; ++i)
    if (bar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   saddr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
// shared-memory matrix descriptor, no swizzle, K-major:
// start address, leading byte offset (between 8-element K groups), stride
// byte offset (between 8-row groups), all in 16-byte units; version 1
__device__ __forceinline__ uint64_t sdesc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor of kind::f16: D F32, A and B BF16, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24
template <int N>
__host__ __device__ constexpr uint32_t idesc_bf16_m128() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(kTile >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          saddr(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 8 BF16 values of v where the matching value of m is positive, else 0
__device__ __forceinline__ uint4 mask8(uint4 v, uint4 m) {
  unsigned* pv = &v.x;
  const unsigned* pm = &m.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bf162 mm = *reinterpret_cast<const bf162*>(&pm[i]);
    unsigned keep = 0;
    if (__low2float(mm) > 0.0f) keep |= 0x0000ffffu;
    if (__high2float(mm) > 0.0f) keep |= 0xffff0000u;
    pv[i] &= keep;
  }
  return v;
}

// pixel slots per staged row (130 used).  Threads store consecutive 16-byte
// groups of a pixel's channels, KC groups per pixel, into rows LBO_A bytes
// apart; the slot count makes the eight stores of a quarter warp hit eight
// different 16-byte bank groups: LBO_A = 64 (KC = 2), 32 (KC = 4) or
// 16 (KC = 8) bytes modulo 128.
template <int KC>
constexpr int slots() {
  return KC == 2 ? 132 : KC == 4 ? 130 : 137;
}

template <int CIN, int COUT>
struct TcShape {
  static constexpr int KC = CIN / 8;               // 16-byte channel groups
  static constexpr int LBO_A = slots<KC>() * 16;   // between channel groups of a staged row
  static constexpr int ROWB = KC * LBO_A;          // bytes per staged row
  static constexpr int LBO_B = COUT * 16;          // between channel groups of a tap's weights
  static constexpr int TAPB = CIN * COUT * 2;      // bytes per tap of weights
  static constexpr int WB = 9 * TAPB;
  static constexpr int OFF_RING = (WB + 127) / 128 * 128;
  static constexpr int OFF_BIAS = OFF_RING + kRing * ROWB;
  static constexpr int OFF_BAR = OFF_BIAS + COUT * 4;
  static constexpr int SMEM = 128 + OFF_BAR + 16;  // + slack to align the base to 128 bytes
  static constexpr unsigned TCOLS = COUT <= 32 ? 32u : 64u;  // TMEM columns (power of 2 >= 32)
  static constexpr int NE = 130 * KC;                        // 16-byte groups of a staged row
  static constexpr int NIT = (NE + kTile - 1) / kTile;       // per thread
};

template <int CIN, int COUT, bool UPS, bool MASK, bool ADD, bool RELU>
__global__ void __launch_bounds__(kTile) k_conv_tc(ConvArgs p, int rows, int* err) {
  using S = TcShape<CIN, COUT>;
  constexpr int KC = S::KC, NE = S::NE, NIT = S::NIT;
  extern __shared__ __align__(128) unsigned char tc_raw[];
  unsigned char* sm = tc_raw + ((128u - (saddr(tc_raw) & 127u)) & 127u);
  unsigned char* ring = sm + S::OFF_RING;
  float* bias = reinterpret_cast<float*>(sm + S::OFF_BIAS);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S::OFF_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + S::OFF_BAR + 8);
  const int t = threadIdx.x, warp = t >> 5;

  // weights [co][tap][ci] -> [tap][ci/8][co][8 ci] (output channel fastest:
  // consecutive threads store consecutive 16-byte groups)
  for (int i = t; i < COUT * 9 * KC; i += kTile) {
    const int co = i % COUT, c = (i / COUT) % KC, tap = i / (COUT * KC);
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(p.wt) + (co * 9 + tap) * KC + c);
    *reinterpret_cast<uint4*>(sm + tap * S::TAPB + c * S::LBO_B + co * 16) = v;
  }
  if (t < COUT) bias[t] = p.bias ? p.bias[t] : 0.0f;
  if (warp == 0) tmem_alloc(tslot, S::TCOLS);
  if (t == 0) bar_init(bar, 1);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  const int H = p.H, W = p.W;
  const int Hi = UPS ? H / 2 : H, Wi = UPS ? W / 2 : W;
  const int nseg = (W + kTile - 1) / kTile, chunks = (H + rows - 1) / rows;
  const int items = p.n * nseg * chunks;
  const unsigned abase = saddr(ring), wbase = saddr(sm);
  constexpr uint32_t IDESC = idesc_bf16_m128<COUT>();
  unsigned phase = 0;
  bool ok = true;

  // Staging of input row yy (full-resolution coordinate, -1..H) of image img
  // for the segment at x0, in two halves: load() issues the global loads into
  // registers, put() stores them into the row's ring slot.  Rows outside the
  // image, pixels outside the row and the ReLU-masked entries are zeros.
  uint4 v[NIT];
  auto load_to = [&](uint4 (&u)[NIT], int img, int x0, int yy) {
#pragma unroll
    for (int k = 0; k < NIT; ++k) {
      const int e = t + k * kTile;
      const int s = e / KC, c = e % KC, x = x0 - 1 + s;
      u[k] = make_uint4(0u, 0u, 0u, 0u);
      if (e < NE && yy >= 0 && yy < H && x >= 0 && x < W) {
        const int yi = UPS ? (yy >> 1) : yy, xi = UPS ? (x >> 1) : x;
        const size_t off = (((size_t)img * Hi + yi) * Wi + xi) * CIN + c * 8;
        u[k] = __ldg(reinterpret_cast<const uint4*>(p.in + off));
        if (MASK) u[k] = mask8(u[k], __ldg(reinterpret_cast<const uint4*>(p.mask + off)));
      }
    }
  };
  auto put_from = [&](const uint4 (&u)[NIT], int yy) {
    unsigned char* dst = ring + ((yy + 1) & (kRing - 1)) * S::ROWB;
#pragma unroll
    for (int k = 0; k < NIT; ++k) {
      const int e = t + k * kTile;
      if (e < NE) *reinterpret_cast<uint4*>(dst + (e % KC) * S::LBO_A + (e / KC) * 16) = u[k];
    }
  };
  auto load = [&](int img, int x0, int yy) { load_to(v, img, x0, yy); };
  auto put = [&](int yy) { put_from(v, yy); };

  for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
    const int ch = item % chunks, seg = (item / chunks) % nseg, img = item / (chunks * nseg);
    const int x0 = seg * kTile, ya = ch * rows, yb = min(H, ya + rows);
    {  // the first tile's three rows: all loads in flight before any store
      uint4 u0[NIT], u1[NIT];
      load_to(u0, img, x0, ya - 1);
      load_to(u1, img, x0, ya);
      load(img, x0, ya + 1);
      put_from(u0, ya - 1);
      put_from(u1, ya);
      put(ya + 1);
    }
    fence_async_smem();
    __syncthreads();
    for (int y = ya; y < yb; ++y) {
      if (t == 0) {
        tc_fence_after();
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
          const int dy = tap / 3, dx = tap % 3;
          const unsigned arow = abase + ((y + dy) & (kRing - 1)) * S::ROWB + dx * 16;
          const unsigned btap = wbase + tap * S::TAPB;
#pragma unroll
          for (int ks = 0; ks < CIN / 16; ++ks) {
            const uint64_t a = sdesc(arow + 2 * ks * S::LBO_A, S::LBO_A, 128);
            const uint64_t b = sdesc(btap + 2 * ks * S::LBO_B, S::LBO_B, 128);
            mma_bf16(tmem, a, b, IDESC, (tap | ks) != 0);
          }
        }
        mma_commit(bar);
      }
      // the next tile's new row: loads in flight during this tile's MMAs and
      // epilogue, stored afterwards into the slot of row y-2 (read by no MMA
      // in flight)
      const bool more = y + 1 < yb;
      if (more) load(img, x0, y + 2);
      const bool got = bar_wait_bounded(bar, phase);
      if (!__syncthreads_and(got)) {
        ok = false;
        break;
      }
      phase ^= 1u;
      tc_fence_after();
      uint32_t r[COUT];
#pragma unroll
      for (int j = 0; j < COUT / 16; ++j)
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + j * 16,
                  *reinterpret_cast<uint32_t(*)[16]>(&r[j * 16]));
      tmem_wait_ld();
      const int x = x0 + t;
      if (x < W) {
        const size_t off = (((size_t)img * H + y) * W + x) * COUT;
#pragma unroll
        for (int g = 0; g < COUT / 8; ++g) {
          float f[8];
#pragma unroll
          for (int k = 0; k < 8; ++k) f[k] = __uint_as_float(r[g * 8 + k]) + bias[g * 8 + k];
          if (ADD) {
            const uint4 a = __ldg(reinterpret_cast<const uint4*>(p.add + off) + g);
            const bf162* ab = reinterpret_cast<const bf162*>(&a);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              f[2 * k] += __low2float(ab[k]);
              f[2 * k + 1] += __high2float(ab[k]);
            }
          }
          if (RELU) {
#pragma unroll
            for (int k = 0; k < 8; ++k) f[k] = fmaxf(f[k], 0.0f);
          }
          uint4 o;
          bf162* ob = reinterpret_cast<bf162*>(&o);
#pragma unroll
          for (int k = 0; k < 4; ++k) ob[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
          *(reinterpret_cast<uint4*>(p.out + off) + g) = o;
        }
      }
      if (more) put(y + 2);
      fence_async_smem();
      tc_fence_before();
      __syncthreads();  // row y+2 staged; this tile's TMEM reads done before the next MMAs
    }
  }
  if (!ok) {
    if (t == 0) atomicExch(err, 1);
    bar_wait_bounded(bar, phase);  // let the MMAs in flight finish (bounded)
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, S::TCOLS);
}

// ---------------------------------------------------------------------------
// The forward ReLU layers (input at full resolution, no mask, no skip add)
// with the staged rows copied by the tensor-memory-access unit: one thread
// issues, per input row, one cp.async.bulk.tensor copy of the 130 pixels
// x0-1 .. x0+128 times all CIN channels straight into the ring slot's
// canonical layout, and the copy completes on the slot's own mbarrier.  The
// tensor map describes the NHWC tensor with its dimensions reordered --
// (8 channels, pixel, channel group, row, image) -- so that a box of
// (8, 130, CIN/8, 1, 1) lands as [channel group][pixel][8 channels]: the
// no-swizzle K-major layout with 16 bytes per pixel and 2080 bytes between
// channel groups.  Coordinates outside the image (the pixel before and after
// the row, the rows above and below it) read as zeros: the convolution's
// padding.  Rows are fetched two tiles ahead (five ring slots: the MMAs of
// tile y read rows y-1 .. y+1, row y+2 is in flight, row y+3 is issued), so
// the threads do no staging at all; they only run the epilogue.
constexpr int kTmaSlots = 5;
constexpr int kTmaAcc = 4;  // TMEM accumulators per CTA (a power of two)
constexpr int kTmaPix = 130;
constexpr int kTmaDrain = 256;                  // epilogue: two warps per TMEM lane quadrant
constexpr int kTmaThreads = kTmaDrain + 32;     // + the warp that copies rows and issues MMAs

template <int CIN, int COUT, int SLOTS = kTmaSlots>
struct TmaShape {
  static constexpr int KC = CIN / 8;
  static constexpr int LBO_A = kTmaPix * 16;                 // between channel groups
  static constexpr int ROW_BYTES = KC * LBO_A;                // one copy
  static constexpr int ROWB = (ROW_BYTES + 127) / 128 * 128;  // slot stride (128-byte aligned)
  static constexpr int LBO_B = COUT * 16;
  static constexpr int TAPB = CIN * COUT * 2;
  static constexpr int WB = 9 * TAPB;
  static constexpr int OFF_RING = (WB + 127) / 128 * 128;
  static constexpr int OFF_BIAS = OFF_RING + SLOTS * ROWB;
  // barriers: full[kTmaAcc] (MMAs of an accumulator done), empty[kTmaAcc]
  // (accumulator drained), one per ring slot (row arrived); then the TMEM
  // address and the abort flag
  static constexpr int OFF_BAR = OFF_BIAS + COUT * 4;
  static constexpr int SMEM = 128 + OFF_BAR + 8 * (2 * kTmaAcc + kTmaSlots) + 16;
  // kTmaAcc accumulators of COUT FP32 columns
  static constexpr unsigned TCOLS = COUT <= 16 ? 64u : COUT <= 32 ? 128u : 256u;
  static_assert(kTmaAcc * COUT <= (int)TCOLS, "accumulators exceed the allocation");
  static constexpr int HALF = COUT / 2;  // columns drained by one warp
};

__device__ __forceinline__ void bar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_row(void* dst, const CUtensorMap* map, int x, int row, int img,
                                        uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(saddr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(x), "r"(0), "r"(row), "r"(img),
      "r"(saddr(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
}

// One waits on an mbarrier phase, bounded, giving up early once another
// thread of the CTA has raised the abort flag; a wait that runs out raises it.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, unsigned parity,
                                              volatile int* abort) {
  for (int i = 0; i < kSpins; ++i) {
    if (bar_try_wait(bar, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  return false;
}
__device__ __forceinline__ void bar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}

// Warp roles.  Warp 8 (one thread) copies the rows by TMA and issues the MMAs
// of tile t into accumulator t mod kTmaAcc (four) as soon as the accumulator
// is drained (its `empty` barrier) and the rows have arrived, then commits
// them to the accumulator's `full` barrier; warps 0-7 wait on `full`, drain
// their quarter of the pixels and half of the channels, and arrive on
// `empty`.  Both roles walk the same items and tiles, so the tensor core runs
// up to three tiles ahead of the epilogue, and no block-wide barrier sits in
// the loop.  The producer waits for MMAs only on a row's first tile: when the
// previous tile is done, the rows below the current one are free, and the
// row SLOTS-2 ahead is copied into the slot of the row two behind.
// UPS (the decoder's first convolutions: nearest upsampling of a
// half-resolution input, then the skip tensor added, no ReLU): the rows,
// segments and copies are those of the half-resolution input, and each
// half-resolution row y gives four tiles, output rows 2y + py and pixels
// 2x + px of one parity (py, px).  Tap (dy, dx) of output pixel
// (2y + py, 2x + px) reads the upsampled input at (2y + py - 1 + dy,
// 2x + px - 1 + dx), which is half-resolution pixel
// (y + ((py - 1 + dy) >> 1), x + ((px - 1 + dx) >> 1)): a shifted window of the
// staged rows like the plain convolution's, with the same products summed
// in the same tap order, and the padding row or column of the upsampled
// input maps to the padding of the half-resolution one.  Four tiles per row
// leave time to copy a row one row ahead, so the ring has four slots there
// (the decoder's 64->32 layer fits two CTAs on an SM), and the epilogue loads
// the next tile's skip values while it finishes the current one.
// CTAs per SM that shared memory allows, as the register bound of the
// kernel: 64-channel layers 1, 32->64 and the 64->32 upsampling 2, 32->32 3,
// 16->32 and the 32->16 upsampling 4
constexpr int tma_ctas(int cin, int cout, bool ups) {
  return (cin == 64 && cout == 64)             ? 1
         : (cout == 64 || (ups && cin == 64)) ? 2
         : (cin == 32 && !ups)                ? 3
                                              : 4;
}

template <int CIN, int COUT, bool UPS>
__global__ void __launch_bounds__(kTmaThreads, tma_ctas(CIN, COUT, UPS))
    k_conv_tma(ConvArgs p, int rows, int* err, const CUtensorMap* map) {
  constexpr int SLOTS = UPS ? 4 : kTmaSlots;  // ring slots; a row is copied SLOTS-2 rows ahead
  using S = TmaShape<CIN, COUT, SLOTS>;
  constexpr int KC = S::KC, HALF = S::HALF;
  constexpr int NSUB = UPS ? 4 : 1;  // tiles per staged row
  extern __shared__ __align__(128) unsigned char tm_raw[];
  unsigned char* sm = tm_raw + ((128u - (saddr(tm_raw) & 127u)) & 127u);
  unsigned char* ring = sm + S::OFF_RING;
  float* bias = reinterpret_cast<float*>(sm + S::OFF_BIAS);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + S::OFF_BAR);
  uint64_t* empty = full + kTmaAcc;
  uint64_t* rbar = full + 2 * kTmaAcc;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(rbar + kTmaSlots);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

  for (int i = t; i < COUT * 9 * KC; i += kTmaThreads) {
    const int co = i % COUT, c = (i / COUT) % KC, tap = i / (COUT * KC);
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(p.wt) + (co * 9 + tap) * KC + c);
    *reinterpret_cast<uint4*>(sm + tap * S::TAPB + c * S::LBO_B + co * 16) = v;
  }
  if (t < COUT) bias[t] = p.bias ? p.bias[t] : 0.0f;
  if (warp == 0) tmem_alloc(tslot, S::TCOLS);
  if (t == 0) {
    for (int k = 0; k < kTmaAcc; ++k) {
      bar_init(full + k, 1);
      bar_init(empty + k, kTmaDrain / 32);  // one arrival per draining warp
    }
    for (int k = 0; k < kTmaSlots; ++k) bar_init(rbar + k, 1);
    *abort = 0;
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  const int H = p.H, W = p.W;
  const int RH = UPS ? H / 2 : H, RW = UPS ? W / 2 : W;  // the staged rows
  const int nseg = (RW + kTile - 1) / kTile, chunks = (RH + rows - 1) / rows;
  const int items = p.n * nseg * chunks;

  if (warp == kTmaDrain / 32) {
    if (lane == 0) {  // ---- rows and MMAs ----
      const unsigned abase = saddr(ring), wbase = saddr(sm);
      constexpr uint32_t IDESC = idesc_bf16_m128<COUT>();
      unsigned rphase = 0u, rpend = 0u;  // per slot: next arrival parity, copy in flight
      unsigned fphase = 0u, ephase = 0u, fpend = 0u;  // per accumulator
      unsigned used = 0u;  // per accumulator: held a tile before
      int tile = 0;        // tiles issued by this CTA (accumulator = tile mod kTmaAcc)
      auto slot_of = [](int yy) { return (yy + 1) % SLOTS; };
      auto fetch = [&](int img, int x0, int yy) {
        const int s = slot_of(yy);
        bar_expect_tx(rbar + s, (unsigned)S::ROW_BYTES);
        tma_row(ring + s * S::ROWB, map, x0 - 1, yy, img, rbar + s);
        rpend |= 1u << s;
      };
      auto arrived = [&](int yy) -> bool {
        const int s = slot_of(yy);
        if (!wait_or_abort(rbar + s, (rphase >> s) & 1u, abort)) return false;
        rphase ^= 1u << s;
        rpend &= ~(1u << s);
        return true;
      };
      // the MMAs committed to accumulator b are done (every commit is
      // accounted for once, here or when the epilogue has drained the
      // accumulator, so the parities stay in step)
      auto retire = [&](int b) -> bool {
        if (!((fpend >> b) & 1u)) return true;
        if (!wait_or_abort(full + b, (fphase >> b) & 1u, abort)) return false;
        fphase ^= 1u << b;
        fpend &= ~(1u << b);
        return true;
      };
      bool go = true;
      for (int item = blockIdx.x; item < items && go; item += gridDim.x) {
        const int ch = item % chunks, seg = (item / chunks) % nseg, img = item / (chunks * nseg);
        const int x0 = seg * kTile, ya = ch * rows, yb = min(RH, ya + rows);
        for (int yy = ya - 1; yy <= ya + SLOTS - 3 && yy <= yb; ++yy) fetch(img, x0, yy);
        go = arrived(ya - 1) && arrived(ya);
        for (int y = ya; y < yb && go; ++y) {
          if (!arrived(y + 1)) { go = false; break; }
          const int s0 = slot_of(y - 1);
          for (int sub = 0; sub < NSUB; ++sub, ++tile) {
            const int b = tile & (kTmaAcc - 1);
            if ((used >> b) & 1u) {  // the epilogue has drained this accumulator
              if (!wait_or_abort(empty + b, (ephase >> b) & 1u, abort)) { go = false; break; }
              ephase ^= 1u << b;
              if ((fpend >> b) & 1u) {  // so its last MMAs are done
                fphase ^= 1u << b;
                fpend &= ~(1u << b);
              }
            }
            tc_fence_after();
            const int py = sub >> 1, px = sub & 1;
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
              const int dy = tap / 3, dx = tap % 3;
              // staged row (0..2 from row y-1) and pixel shift of the tap
              const int ry = UPS ? 1 + ((py - 1 + dy) >> 1) : dy;
              const int rx = UPS ? 1 + ((px - 1 + dx) >> 1) : dx;
              const int slot = s0 + ry < SLOTS ? s0 + ry : s0 + ry - SLOTS;
              const unsigned arow = abase + slot * S::ROWB + rx * 16;
              const unsigned btap = wbase + tap * S::TAPB;
#pragma unroll
              for (int ks = 0; ks < CIN / 16; ++ks) {
                const uint64_t a = sdesc(arow + 2 * ks * S::LBO_A, S::LBO_A, 128);
                const uint64_t bb = sdesc(btap + 2 * ks * S::LBO_B, S::LBO_B, 128);
                mma_bf16(tmem + b * COUT, a, bb, IDESC, (tap | ks) != 0);
              }
            }
            mma_commit(full + b);
            used |= 1u << b;
            fpend |= 1u << b;
            // on the row's first tile: the previous tile's MMAs (queued ahead
            // of these) done finishes row y-1's tiles, so rows up to y-2 are
            // free and row y+SLOTS-2 takes the slot of row y-2
            if (sub == 0) {
              if (!retire((tile - 1) & (kTmaAcc - 1))) { go = false; break; }
              if (y + SLOTS - 2 <= yb) fetch(img, x0, y + SLOTS - 2);
            }
          }
        }
        // the item's last MMAs are done before the next item refills the slots
        for (int b = 0; b < kTmaAcc && go; ++b) go = retire(b);
      }
      if (!go) {
        *abort = 1;
        atomicExch(err, 1);
        // let the copies and MMAs in flight land (bounded) before the memory goes
        for (int s = 0; s < kTmaSlots; ++s)
          if ((rpend >> s) & 1u) bar_wait_bounded(rbar + s, (rphase >> s) & 1u);
        for (int b = 0; b < kTmaAcc; ++b)
          if ((fpend >> b) & 1u) bar_wait_bounded(full + b, (fphase >> b) & 1u);
      }
    }
  } else {  // ---- epilogue: warps 0-7 ----
    const int quad = warp & 3, half = warp >> 2;  // TMEM lanes 32 quad .., columns half * HALF ..
    float bv[HALF];
#pragma unroll
    for (int k = 0; k < HALF; ++k) bv[k] = bias[half * HALF + k];
    // this CTA's tiles in issue order: item, staged row y, parity sub
    struct Pos {
      int item, img, x0, y, yb, sub;
    };
    auto enter = [&](Pos& q) {  // first tile of item q.item
      const int ch = q.item % chunks, seg = (q.item / chunks) % nseg;
      q.img = q.item / (chunks * nseg);
      q.x0 = seg * kTile;
      q.y = ch * rows;
      q.yb = min(RH, q.y + rows);
      q.sub = 0;
    };
    auto advance = [&](Pos& q) {
      if (++q.sub < NSUB) return;
      q.sub = 0;
      if (++q.y < q.yb) return;
      q.item += gridDim.x;
      if (q.item < items) enter(q);
    };
    // output element offset of this thread's pixel in tile q (-1: beyond the row)
    auto out_off = [&](const Pos& q) -> long long {
      const int xs = q.x0 + quad * 32 + lane;  // staged pixel of this thread
      if (xs >= RW) return -1;
      const int oy = UPS ? 2 * q.y + (q.sub >> 1) : q.y, ox = UPS ? 2 * xs + (q.sub & 1) : xs;
      return (((long long)q.img * H + oy) * W + ox) * COUT + half * HALF;
    };
    uint4 skip[UPS ? HALF / 8 : 1];
    auto load_skip = [&](const Pos& q) {
      if constexpr (UPS) {
        const long long off = out_off(q);
        if (off >= 0) {
#pragma unroll
          for (int g = 0; g < HALF / 8; ++g)
            skip[g] = __ldg(reinterpret_cast<const uint4*>(p.add + off) + g);
        }
      }
    };
    unsigned fphase = 0u;
    Pos pos{};
    pos.item = blockIdx.x;
    if (pos.item < items) {
      enter(pos);
      load_skip(pos);
    }
    for (int tile = 0; pos.item < items; ++tile) {
      const int b = tile & (kTmaAcc - 1);
      if (!wait_or_abort(full + b, (fphase >> b) & 1u, abort)) break;
      fphase ^= 1u << b;
      tc_fence_after();
      uint32_t r[HALF];
      const uint32_t ta = tmem + ((uint32_t)(quad * 32) << 16) + b * COUT + half * HALF;
      if constexpr (HALF == 8) {
        tmem_ld8(ta, *reinterpret_cast<uint32_t(*)[8]>(&r[0]));
      } else {
#pragma unroll
        for (int j = 0; j < HALF / 16; ++j)
          tmem_ld16(ta + j * 16, *reinterpret_cast<uint32_t(*)[16]>(&r[j * 16]));
      }
      tmem_wait_ld();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) bar_arrive(empty + b);  // the accumulator is free again
      const long long off = out_off(pos);
      uint4 cur[UPS ? HALF / 8 : 1];
#pragma unroll
      for (int g = 0; g < (UPS ? HALF / 8 : 1); ++g) cur[g] = skip[g];
      advance(pos);
      if (pos.item < items) load_skip(pos);  // in flight while this tile is stored
      if (off >= 0) {
#pragma unroll
        for (int g = 0; g < HALF / 8; ++g) {
          float f[8];
#pragma unroll
          for (int k = 0; k < 8; ++k) f[k] = __uint_as_float(r[g * 8 + k]) + bv[g * 8 + k];
          if constexpr (UPS) {  // skip tensor added, no ReLU
            const bf162* ab = reinterpret_cast<const bf162*>(&cur[g]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              f[2 * k] += __low2float(ab[k]);
              f[2 * k + 1] += __high2float(ab[k]);
            }
          } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) f[k] = fmaxf(f[k], 0.0f);
          }
          uint4 o;
          bf162* ob = reinterpret_cast<bf162*>(&o);
#pragma unroll
          for (int k = 0; k < 4; ++k) ob[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
          *(reinterpret_cast<uint4*>(p.out + off) + g) = o;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, S::TCOLS);
}

// resident CTAs per SM from the kernel's registers and shared memory (the
// occupancy query does not count these kernels correctly) and the tensor
// memory: 512 columns per SM
template <class K>
int resident_ctas(K k, int smem, unsigned tcols, int threads = kTile) {
  cudaFuncAttributes fa{};
  int dev = 0, smem_sm = 0, resv = 0, regs_sm = 0, thr_sm = 0;
  if (cudaFuncGetAttributes(&fa, k) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) !=
          cudaSuccess ||
      cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev) !=
          cudaSuccess ||
      cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) !=
          cudaSuccess ||
      cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess)
    return 0;
  const int per_smem = smem_sm / (smem + fa.sharedSizeBytes + resv);
  const int warp_regs = (fa.numRegs * 32 + 255) / 256 * 256;  // allocation unit: 256 per warp
  const int per_regs = regs_sm / (warp_regs * (threads / 32));
  const int per_thr = thr_sm / threads;
  const int per_tmem = 512 / (int)tcols;
  int o = per_smem;
  if (per_regs < o) o = per_regs;
  if (per_thr < o) o = per_thr;
  if (per_tmem < o) o = per_tmem;
  return o;
}

template <int CIN, int COUT, bool UPS, bool MASK, bool ADD, bool RELU>
int launch_tc(const ConvArgs& a, int sms, int* err, cudaStream_t s) {
  using S = TcShape<CIN, COUT>;
  auto k = k_conv_tc<CIN, COUT, UPS, MASK, ADD, RELU>;
  static const int occ = [k] {
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM) !=
        cudaSuccess)
      return 0;
    return resident_ctas(k, S::SMEM, S::TCOLS);
  }();
  if (occ <= 0) return -1;
  const long long nseg = (a.W + kTile - 1) / kTile;
  const long long slots = (long long)sms * occ;
  const long long total_rows = (long long)a.n * nseg * a.H;
  int rows = (int)((total_rows + slots - 1) / slots);
  if (rows < 1) rows = 1;
  const long long items = (long long)a.n * nseg * ((a.H + rows - 1) / rows);
  const int grid = (int)(items < slots ? items : slots);
  k<<<grid, kTile, S::SMEM, s>>>(a, rows, err);
  ++g_launches;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int CIN, int COUT, bool UPS>
int launch_tma(const ConvArgs& a, int sms, int* err, const CUtensorMap* map, cudaStream_t s) {
  using S = TmaShape<CIN, COUT, UPS ? 4 : kTmaSlots>;
  auto k = k_conv_tma<CIN, COUT, UPS>;
  static const int occ = [k] {
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM) !=
        cudaSuccess)
      return 0;
    return resident_ctas(k, S::SMEM, S::TCOLS, kTmaThreads);
  }();
  if (occ <= 0) return -1;
  // the staged rows: the input's (half the output's when upsampling)
  const int RH = UPS ? a.H / 2 : a.H, RW = UPS ? a.W / 2 : a.W;
  const long long nseg = (RW + kTile - 1) / kTile;
  const long long slots = (long long)sms * occ;
  const long long total_rows = (long long)a.n * nseg * RH;
  int rows = (int)((total_rows + slots - 1) / slots);
  if (rows < 1) rows = 1;
  const long long items = (long long)a.n * nseg * ((RH + rows - 1) / rows);
  const int grid = (int)(items < slots ? items : slots);
  k<<<grid, kTmaThreads, S::SMEM, s>>>(a, rows, err, map);
  ++g_launches;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <int CI, int CO>
constexpr bool up_pair() {
  return (CI == 64 && CO == 64) || (CI == 64 && CO == 32) || (CI == 32 && CO == 16);
}
template <int CI, int CO>
constexpr bool relu_pair() {
  return (CI == 16 && CO == 16) || (CI == 16 && CO == 32) || (CI == 32 && CO == 32) ||
         (CI == 32 && CO == 64) || (CI == 64 && CO == 64);
}

// forward: upsampling decoder layer (+ skip add) or conv + ReLU;
// backward (input gradient): CIN/COUT are the layer's COUT/CIN, the output
// gradient masked by the ReLU output for ReLU layers
template <int CI, int CO>
int dispatch_pair(const ConvArgs& a, bool ups, bool bwd, bool mask, int sms, int* err,
                  const CUtensorMap* map, cudaStream_t s) {
  if (!bwd) {
    if constexpr (up_pair<CI, CO>()) {
      if (ups && map) return launch_tma<CI, CO, true>(a, sms, err, map, s);
      if (ups) return launch_tc<CI, CO, true, false, true, false>(a, sms, err, s);
    }
    if constexpr (relu_pair<CI, CO>()) {
      // 16 -> 16: nine small MMAs per tile; the warp roles run these layers
      // no faster than the thread staging (67 against 66 us per 2048^2
      // layer with four accumulators, 91 with two), so they keep it
      if constexpr (CI > 16 || CO > 16)
        if (!ups && map) return launch_tma<CI, CO, false>(a, sms, err, map, s);
      if (!ups) return launch_tc<CI, CO, false, false, false, true>(a, sms, err, s);
    }
    return -1;
  }
  if constexpr (relu_pair<CO, CI>())
    if (mask) return launch_tc<CI, CO, false, true, false, false>(a, sms, err, s);
  if constexpr (up_pair<CO, CI>())
    if (!mask) return launch_tc<CI, CO, false, false, false, false>(a, sms, err, s);
  return -1;
}

}  // namespace

int conv_tc(int cin, int cout, const ConvArgs& a, bool ups, bool bwd, bool mask, int sms,
            int* err, const CUtensorMap* map, cudaStream_t s) {
#define SCF_TC(CI, CO) \
  if (cin == CI && cout == CO) return dispatch_pair<CI, CO>(a, ups, bwd, mask, sms, err, map, s);
  SCF_TC(16, 16) SCF_TC(16, 32) SCF_TC(32, 16) SCF_TC(32, 32) SCF_TC(32, 64) SCF_TC(64, 32)
  SCF_TC(64, 64)
#undef SCF_TC
  return -1;
}

namespace {
typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                             const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                             const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                             CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeFn encoder() {
  static EncodeFn fn = [] {
    void* q = nullptr;
    cudaDriverEntryPointQueryResult r = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &q, 12000, cudaEnableDefault,
                                         &r) != cudaSuccess ||
        r != cudaDriverEntryPointSuccess)
      return (EncodeFn) nullptr;
    return reinterpret_cast<EncodeFn>(q);
  }();
  return fn;
}
}  // namespace

int conv_tma_map(CUtensorMap* m, const void* in, int n, int H, int W, int cin) {
  EncodeFn fn = encoder();
  if (!fn || (reinterpret_cast<uintptr_t>(in) & 15) || cin % 16 || W < 1 || H < 1 || n < 1)
    return -1;
  const cuuint64_t e = 2;  // BF16
  // (8 channels, pixel, channel group, row, image)
  const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)(cin / 8), (cuuint64_t)H,
                              (cuuint64_t)n};
  const cuuint64_t strides[4] = {(cuuint64_t)cin * e, 16, (cuuint64_t)W * cin * e,
                                 (cuuint64_t)H * W * cin * e};
  const cuuint32_t box[5] = {8, (cuuint32_t)kTmaPix, (cuuint32_t)(cin / 8), 1, 1};
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(in), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
             ? 0
             : -1;
}

}  // namespace scf
