// scf_unet.cu -- kernels and host driver of the learned preconditioner (the
// U-Net of include/scf_unet.h): BF16 3x3 convolutions on the tensor cores
// (mma.sync m16n8k16, FP32 accumulation) for the forward pass, the input
// gradient and the weight gradient; pooling, the 1x1 head, the loss and Adam.
//
// Activations are NHWC BF16 with 16, 32 or 64 channels.  A convolution is an
// implicit GEMM: M = output pixels (tiles of 8 x 16), N = output channels,
// K = 9 taps x input channels.  One CTA (4 warps) keeps the whole weight
// tensor of the layer in shared memory and loops over output tiles; per tile
// it stages the input with a one-pixel halo (optionally read at half
// resolution for nearest upsampling, or masked by a ReLU output for the
// backward pass) and each warp computes two rows of 16 pixels for all output
// channels from ldmatrix fragments.  The input gradient is the same kernel
// with the weights flipped and transposed; the weight gradient reduces over
// pixels with ldmatrix.trans fragments, one tap per CTA row of the grid,
// FP32 atomics at the end.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/scf_unet.h"
#include "scf_unet.cuh"

namespace scf {
extern thread_local long long g_launches;  // defined with the multigrid launchers
inline void note_launch() { ++g_launches; }
}  // namespace scf

namespace scf {
namespace {

using bf16 = __nv_bfloat16;
using bf162 = __nv_bfloat162;

constexpr int TH = 8, TW = 16, NTH = 128;  // output tile, threads per CTA

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2_t(unsigned& r0, unsigned& r1, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
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

using ConvP = ConvArgs;

template <int CIN, int COUT>
constexpr int conv_smem() {
  return (COUT * (9 * CIN + 8) + (TH + 2) * (TW + 2) * (CIN + 8)) * 2;
}

template <int CIN, int COUT, bool UPS, bool MASK, bool ADD, bool RELU>
__global__ void __launch_bounds__(NTH) k_conv(ConvP p) {
  extern __shared__ __align__(16) unsigned char csm[];
  constexpr int WS = 9 * CIN + 8;  // weight row stride (elements): conflict-free ldmatrix
  constexpr int XS = CIN + 8;      // staged pixel stride
  bf16* Wsm = reinterpret_cast<bf16*>(csm);
  bf16* Xsm = Wsm + COUT * WS;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  constexpr int WV = 9 * CIN / 8;  // 16-byte vectors per weight row
  for (int i = t; i < COUT * WV; i += NTH) {
    const int row = i / WV, c = i % WV;
    *reinterpret_cast<uint4*>(Wsm + row * WS + c * 8) =
        __ldg(reinterpret_cast<const uint4*>(p.wt) + i);
  }
  const int txn = (p.W + TW - 1) / TW, tyn = (p.H + TH - 1) / TH;
  const int ntiles = txn * tyn * p.n;
  const int Hi = UPS ? p.H / 2 : p.H, Wi = UPS ? p.W / 2 : p.W;
  constexpr int C8 = CIN / 8;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int img = tile / (txn * tyn), rem = tile % (txn * tyn);
    const int y0 = (rem / txn) * TH, x0 = (rem % txn) * TW;
    __syncthreads();  // weights stored; the previous tile's fragments read
    for (int i = t; i < (TH + 2) * (TW + 2) * C8; i += NTH) {
      const int c = i % C8, pix = i / C8;
      const int ty = pix / (TW + 2), tx = pix % (TW + 2);
      const int y = y0 + ty - 1, x = x0 + tx - 1;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (y >= 0 && y < p.H && x >= 0 && x < p.W) {
        const int yi = UPS ? (y >> 1) : y, xi = UPS ? (x >> 1) : x;
        const size_t off = (((size_t)img * Hi + yi) * Wi + xi) * CIN + c * 8;
        v = __ldg(reinterpret_cast<const uint4*>(p.in + off));
        if (MASK) v = mask8(v, __ldg(reinterpret_cast<const uint4*>(p.mask + off)));
      }
      *reinterpret_cast<uint4*>(Xsm + pix * XS + c * 8) = v;
    }
    __syncthreads();
    float acc[2][COUT / 8][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < COUT / 8; ++b)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.0f;
    const int apx = (lane & 7) + ((lane >> 3) & 1) * 8, akh = lane >> 4;
    const int bn = (lane >> 4) * 8 + (lane & 7), bkh = (lane >> 3) & 1;
#pragma unroll 1
    for (int tap = 0; tap < 9; ++tap) {
      const int dy = tap / 3, dx = tap % 3;
#pragma unroll
      for (int kc = 0; kc < CIN / 16; ++kc) {
        unsigned a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          const int row = warp * 2 + mt;
          ldsm_x4(a[mt], Xsm + ((row + dy) * (TW + 2) + apx + dx) * XS + kc * 16 + akh * 8);
        }
#pragma unroll
        for (int np = 0; np < COUT / 16; ++np) {
          unsigned b[4];
          ldsm_x4(b, Wsm + (np * 16 + bn) * WS + tap * CIN + kc * 16 + bkh * 8);
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            mma16816(acc[mt][2 * np], a[mt], b[0], b[1]);
            mma16816(acc[mt][2 * np + 1], a[mt], b[2], b[3]);
          }
        }
      }
    }
    const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const int y = y0 + warp * 2 + mt;
#pragma unroll
      for (int nt = 0; nt < COUT / 8; ++nt) {
        const int co = nt * 8 + tig * 2;
        const float b0 = p.bias ? p.bias[co] : 0.0f, b1 = p.bias ? p.bias[co + 1] : 0.0f;
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
          const int x = x0 + gid + hf * 8;
          if (y < p.H && x < p.W) {
            float v0 = acc[mt][nt][2 * hf] + b0, v1 = acc[mt][nt][2 * hf + 1] + b1;
            const size_t off = (((size_t)img * p.H + y) * p.W + x) * COUT + co;
            if (ADD) {
              const bf162 ad = *reinterpret_cast<const bf162*>(p.add + off);
              v0 += __low2float(ad);
              v1 += __high2float(ad);
            }
            if (RELU) {
              v0 = fmaxf(v0, 0.0f);
              v1 = fmaxf(v1, 0.0f);
            }
            *reinterpret_cast<bf162*>(p.out + off) = __floats2bfloat162_rn(v0, v1);
          }
        }
      }
    }
  }
}

struct WgP {
  const bf16* dy;  // [n][H][W][COUT]: gradient of the layer's output
  const bf16* y;   // RELU: the layer's output (mask)
  const bf16* x;   // the layer's input [n][Hi][Wi][CIN]
  float* dw;       // [COUT][9][CIN], accumulated
  float* db;       // [COUT], accumulated by the tap-0 CTAs
  int n, H, W;
};

template <int CIN, int COUT>
constexpr int wgrad_smem() {
  return (TH * TW * (COUT + 8) + TH * TW * (CIN + 8)) * 2;
}

// dW[co][tap][ci] += sum_p dy'[p][co] x[p + tap][ci]; dy' = dy masked by
// y > 0 for ReLU layers.  Grid: (CTAs, 9 taps); each CTA loops over tiles.
template <int CIN, int COUT, bool UPS, bool RELU>
__global__ void __launch_bounds__(NTH) k_wgrad(WgP p) {
  extern __shared__ __align__(16) unsigned char wsm[];
  constexpr int DS = COUT + 8, XS = CIN + 8;
  bf16* Dsm = reinterpret_cast<bf16*>(wsm);
  bf16* Xsm = Dsm + TH * TW * DS;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int tap = blockIdx.y, oy = tap / 3 - 1, ox = tap % 3 - 1;
  constexpr int MT = COUT / 16, NT = CIN / 8, ITEMS = MT * NT;
  constexpr int IPW = (ITEMS + 3) / 4;
  float acc[IPW][4];
#pragma unroll
  for (int j = 0; j < IPW; ++j)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[j][c] = 0.0f;
  float bsum = 0.0f;
  const int txn = (p.W + TW - 1) / TW, tyn = (p.H + TH - 1) / TH;
  const int ntiles = txn * tyn * p.n;
  const int Hi = UPS ? p.H / 2 : p.H, Wi = UPS ? p.W / 2 : p.W;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int img = tile / (txn * tyn), rem = tile % (txn * tyn);
    const int y0 = (rem / txn) * TH, x0 = (rem % txn) * TW;
    __syncthreads();
    for (int i = t; i < TH * TW * (COUT / 8); i += NTH) {
      const int c = i % (COUT / 8), pix = i / (COUT / 8);
      const int y = y0 + pix / TW, x = x0 + pix % TW;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (y < p.H && x < p.W) {
        const size_t off = (((size_t)img * p.H + y) * p.W + x) * COUT + c * 8;
        v = __ldg(reinterpret_cast<const uint4*>(p.dy + off));
        if (RELU) v = mask8(v, __ldg(reinterpret_cast<const uint4*>(p.y + off)));
      }
      *reinterpret_cast<uint4*>(Dsm + pix * DS + c * 8) = v;
    }
    for (int i = t; i < TH * TW * (CIN / 8); i += NTH) {
      const int c = i % (CIN / 8), pix = i / (CIN / 8);
      const int y = y0 + pix / TW + oy, x = x0 + pix % TW + ox;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (y0 + pix / TW < p.H && x0 + pix % TW < p.W && y >= 0 && y < p.H && x >= 0 &&
          x < p.W) {
        const int yi = UPS ? (y >> 1) : y, xi = UPS ? (x >> 1) : x;
        const size_t off = (((size_t)img * Hi + yi) * Wi + xi) * CIN + c * 8;
        v = __ldg(reinterpret_cast<const uint4*>(p.x + off));
      }
      *reinterpret_cast<uint4*>(Xsm + pix * XS + c * 8) = v;
    }
    __syncthreads();
#pragma unroll 1
    for (int ks = 0; ks < TH * TW / 16; ++ks) {
      const int ap = ks * 16 + (lane & 7) + ((lane >> 4) & 1) * 8;
      const int aco = ((lane >> 3) & 1) * 8;
      const int bp = ks * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;
#pragma unroll
      for (int j = 0; j < IPW; ++j) {
        const int item = warp + 4 * j;
        if (item < ITEMS) {
          const int mt = item / NT, nt = item % NT;
          unsigned a[4];
          ldsm_x4_t(a, Dsm + ap * DS + mt * 16 + aco);
          unsigned b0, b1;
          ldsm_x2_t(b0, b1, Xsm + bp * XS + nt * 8);
          mma16816(acc[j], a, b0, b1);
        }
      }
    }
    if (tap == 0 && t < COUT)
      for (int q = 0; q < TH * TW; ++q) bsum += __bfloat162float(Dsm[q * DS + t]);
  }
  const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int j = 0; j < IPW; ++j) {
    const int item = warp + 4 * j;
    if (item < ITEMS) {
      const int mt = item / NT, nt = item % NT;
      const int co = mt * 16 + gid, ci = nt * 8 + tig * 2;
      atomicAdd(&p.dw[((size_t)co * 9 + tap) * CIN + ci], acc[j][0]);
      atomicAdd(&p.dw[((size_t)co * 9 + tap) * CIN + ci + 1], acc[j][1]);
      atomicAdd(&p.dw[((size_t)(co + 8) * 9 + tap) * CIN + ci], acc[j][2]);
      atomicAdd(&p.dw[((size_t)(co + 8) * 9 + tap) * CIN + ci + 1], acc[j][3]);
    }
  }
  if (tap == 0 && t < COUT) atomicAdd(&p.db[t], bsum);
}

// 2x2 mean (fwd) of NHWC BF16, C multiple of 8
__global__ void k_pool(const bf16* __restrict__ in, bf16* __restrict__ out, int n, int H, int W,
                       int C) {
  const int Ho = H / 2, Wo = W / 2, C8 = C / 8;
  const size_t total = (size_t)n * Ho * Wo * C8;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C8);
    size_t q = i / C8;
    const int x = (int)(q % Wo);
    q /= Wo;
    const int y = (int)(q % Ho);
    const int img = (int)(q / Ho);
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(
                                  in + (((size_t)img * H + 2 * y + dy) * W + 2 * x + dx) * C) +
                              c);
        const bf162* h = reinterpret_cast<const bf162*>(&v);
        for (int k = 0; k < 4; ++k) {
          s[2 * k] += __low2float(h[k]);
          s[2 * k + 1] += __high2float(h[k]);
        }
      }
    uint4 o;
    bf162* oh = reinterpret_cast<bf162*>(&o);
    for (int k = 0; k < 4; ++k) oh[k] = __floats2bfloat162_rn(0.25f * s[2 * k], 0.25f * s[2 * k + 1]);
    reinterpret_cast<uint4*>(out + (((size_t)img * Ho + y) * Wo + x) * C)[c] = o;
  }
}

// 2x2 sum (gradient of nearest upsampling) of NHWC BF16
__global__ void k_sumpool(const bf16* __restrict__ in, bf16* __restrict__ out, int n, int H,
                          int W, int C) {
  const int Ho = H / 2, Wo = W / 2, C8 = C / 8;
  const size_t total = (size_t)n * Ho * Wo * C8;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C8);
    size_t q = i / C8;
    const int x = (int)(q % Wo);
    q /= Wo;
    const int y = (int)(q % Ho);
    const int img = (int)(q / Ho);
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(
                                  in + (((size_t)img * H + 2 * y + dy) * W + 2 * x + dx) * C) +
                              c);
        const bf162* h = reinterpret_cast<const bf162*>(&v);
        for (int k = 0; k < 4; ++k) {
          s[2 * k] += __low2float(h[k]);
          s[2 * k + 1] += __high2float(h[k]);
        }
      }
    uint4 o;
    bf162* oh = reinterpret_cast<bf162*>(&o);
    for (int k = 0; k < 4; ++k) oh[k] = __floats2bfloat162_rn(s[2 * k], s[2 * k + 1]);
    reinterpret_cast<uint4*>(out + (((size_t)img * Ho + y) * Wo + x) * C)[c] = o;
  }
}

// out = skip + 0.25 * coarse(parent): gradient of a pooled tensor plus its skip
__global__ void k_unpool_add(const bf16* __restrict__ skip, const bf16* __restrict__ coarse,
                             bf16* __restrict__ out, int n, int H, int W, int C) {
  const int C8 = C / 8;
  const size_t total = (size_t)n * H * W * C8;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C8);
    size_t q = i / C8;
    const int x = (int)(q % W);
    q /= W;
    const int y = (int)(q % H);
    const int img = (int)(q / H);
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(skip) + i);
    const uint4 b = __ldg(reinterpret_cast<const uint4*>(
                              coarse + (((size_t)img * (H / 2) + y / 2) * (W / 2) + x / 2) * C) +
                          c);
    const bf162* ha = reinterpret_cast<const bf162*>(&a);
    const bf162* hb = reinterpret_cast<const bf162*>(&b);
    uint4 o;
    bf162* oh = reinterpret_cast<bf162*>(&o);
    for (int k = 0; k < 4; ++k)
      oh[k] = __floats2bfloat162_rn(__low2float(ha[k]) + 0.25f * __low2float(hb[k]),
                                    __high2float(ha[k]) + 0.25f * __high2float(hb[k]));
    reinterpret_cast<uint4*>(out)[i] = o;
  }
}

// z = w . d0 + b (16 channels -> 1)
__global__ void k_head(const bf16* __restrict__ d0, const float* __restrict__ hw, size_t np,
                       float* __restrict__ z) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < np;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint4* v = reinterpret_cast<const uint4*>(d0 + i * 16);
    float s = hw[16];
    for (int h = 0; h < 2; ++h) {
      const uint4 u = __ldg(v + h);
      const bf162* e = reinterpret_cast<const bf162*>(&u);
      for (int k = 0; k < 4; ++k)
        s = fmaf(__low2float(e[k]), hw[h * 8 + 2 * k], fmaf(__high2float(e[k]), hw[h * 8 + 2 * k + 1], s));
    }
    z[i] = s;
  }
}

// backward of the head: g_d0 = dz w; dw += sum dz d0; db += sum dz
__global__ void k_head_bwd(const bf16* __restrict__ d0, const float* __restrict__ hw,
                           const float* __restrict__ dz, size_t np, bf16* __restrict__ gd0,
                           float* __restrict__ dhw) {
  float acc[17];
  for (int k = 0; k < 17; ++k) acc[k] = 0.0f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < np;
       i += (size_t)gridDim.x * blockDim.x) {
    const float g = dz[i];
    const uint4* v = reinterpret_cast<const uint4*>(d0 + i * 16);
    uint4 o[2];
    for (int h = 0; h < 2; ++h) {
      const uint4 u = __ldg(v + h);
      const bf162* e = reinterpret_cast<const bf162*>(&u);
      bf162* oe = reinterpret_cast<bf162*>(&o[h]);
      for (int k = 0; k < 4; ++k) {
        const int c = h * 8 + 2 * k;
        acc[c] = fmaf(g, __low2float(e[k]), acc[c]);
        acc[c + 1] = fmaf(g, __high2float(e[k]), acc[c + 1]);
        oe[k] = __floats2bfloat162_rn(g * hw[c], g * hw[c + 1]);
      }
    }
    acc[16] += g;
    reinterpret_cast<uint4*>(gd0 + i * 16)[0] = o[0];
    reinterpret_cast<uint4*>(gd0 + i * 16)[1] = o[1];
  }
  for (int k = 0; k < 17; ++k) {
    float s = acc[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&dhw[k], s);
  }
}

// sum over cells with an unknown of (r/dg)^2 and their count, image-wise
__global__ void k_feat_sums(int nx, int ny, int ld, const double* __restrict__ r,
                            const double* __restrict__ dg, float* __restrict__ sums) {
  float s = 0.0f, c = 0.0f;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < (size_t)nx * ny;
       q += (size_t)gridDim.x * blockDim.x) {
    const size_t k = (q / nx) * ld + q % nx;
    const double d = dg[k];
    if (d > 0.0) {
      const float q = (float)(r[k] / d);
      s = fmaf(q, q, s);
      c += 1.0f;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&sums[0], s);
    atomicAdd(&sums[1], c);
  }
}

// input features of image img (see include/scf_unet.h) and sigma; cell
// (x, y) of the operator arrays is at y * ld + x
__global__ void k_features(int nx, int ny, int ld, const double* __restrict__ r,
                           const double* __restrict__ cE, const double* __restrict__ cN,
                           const double* __restrict__ dg, const float* __restrict__ sums,
                           float* __restrict__ sigma_out, bf16* __restrict__ img, int H, int W) {
  const float sig = sums[1] > 0.0f && sums[0] > 0.0f ? sqrtf(sums[0] / sums[1]) : 1.0f;
  if (blockIdx.x == 0 && threadIdx.x == 0 && sigma_out) *sigma_out = sig;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < (size_t)H * W;
       q += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(q % W), y = (int)(q / W);
    float f[5] = {0, 0, 0, 0, 0};
    if (x < nx && y < ny) {
      const size_t k = (size_t)y * ld + x;
      const double d = dg[k];
      if (d > 0.0) {
        const double inv = 1.0 / d;
        f[0] = (float)(r[k] * inv) / sig;
        f[1] = (float)(cE[k] * inv);
        f[2] = x > 0 ? (float)(cE[k - 1] * inv) : 0.0f;
        f[3] = (float)(cN[k] * inv);
        f[4] = y > 0 ? (float)(cN[k - ld] * inv) : 0.0f;
      }
    }
    uint4 o[2];
    bf162* h = reinterpret_cast<bf162*>(o);
    h[0] = __floats2bfloat162_rn(f[0], f[1]);
    h[1] = __floats2bfloat162_rn(f[2], f[3]);
    h[2] = __floats2bfloat162_rn(f[4], 0.0f);
    for (int k = 3; k < 8; ++k) h[k] = __floats2bfloat162_rn(0.0f, 0.0f);
    reinterpret_cast<uint4*>(img + q * 16)[0] = o[0];
    reinterpret_cast<uint4*>(img + q * 16)[1] = o[1];
  }
}

// x[g] = sigma * z(ix, iy) on cells with dg > 0 (padded level layout), else 0
template <class XT>
__global__ void k_correction(int nx, int ny, int pitch, int W, const double* __restrict__ dg,
                             const float* __restrict__ sigma, const float* __restrict__ z,
                             XT* __restrict__ x) {
  const float s = *sigma;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < (size_t)nx * ny;
       q += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(q % nx), iy = (int)(q / nx);
    const size_t g = (size_t)iy * pitch + ix;
    x[g] = dg[g] > 0.0 ? (XT)(s * z[(size_t)iy * W + ix]) : XT(0);
  }
}

// per image: sum of t^2 and of (z - t)^2 over the mask
__global__ void k_loss_sums(const float* __restrict__ z, const float* __restrict__ t,
                            const unsigned char* __restrict__ mask, size_t hw,
                            float* __restrict__ sums) {
  const int img = blockIdx.y;
  float st = 0.0f, se = 0.0f;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < hw;
       q += (size_t)gridDim.x * blockDim.x) {
    const size_t i = (size_t)img * hw + q;
    if (mask[i]) {
      const float d = z[i] - t[i];
      st = fmaf(t[i], t[i], st);
      se = fmaf(d, d, se);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    st += __shfl_down_sync(0xffffffffu, st, o);
    se += __shfl_down_sync(0xffffffffu, se, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&sums[2 * img], st);
    atomicAdd(&sums[2 * img + 1], se);
  }
}

__global__ void k_loss_grad(const float* __restrict__ z, const float* __restrict__ t,
                            const unsigned char* __restrict__ mask, size_t hw,
                            const float* __restrict__ sums, float* __restrict__ dz) {
  const int img = blockIdx.y;
  const float tt = sums[2 * img];
  const float sc = tt > 0.0f ? 2.0f / tt : 0.0f;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < hw;
       q += (size_t)gridDim.x * blockDim.x) {
    const size_t i = (size_t)img * hw + q;
    dz[i] = mask[i] ? sc * (z[i] - t[i]) : 0.0f;
  }
}

__global__ void k_loss_total(const float* __restrict__ sums, int n, float* __restrict__ out) {
  float s = 0.0f;
  for (int i = 0; i < n; ++i) s += sums[2 * i] > 0.0f ? sums[2 * i + 1] / sums[2 * i] : 0.0f;
  *out = s;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// BF16 weights [co][tap][ci] and the flipped transposes [ci][8 - tap][co]
__global__ void k_weights(const float* __restrict__ w, int cin, int cout, bf16* __restrict__ wb,
                          bf16* __restrict__ wt) {
  const int n = cout * 9 * cin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ci = i % cin, tap = (i / cin) % 9, co = i / (9 * cin);
    const bf16 b = __float2bfloat16_rn(w[i]);
    wb[i] = b;
    wt[((size_t)ci * 9 + (8 - tap)) * cout + co] = b;
  }
}

std::vector<UNetLayer> make_layers() {
  // cin, cout, level, ups, relu, skip
  struct D { int cin, cout, level; bool ups, relu; int skip; };
  const D d[] = {{16, 16, 0, false, true, -1}, {16, 16, 0, false, true, -1},
                 {16, 32, 1, false, true, -1}, {32, 32, 1, false, true, -1},
                 {32, 64, 2, false, true, -1}, {64, 64, 2, false, true, -1},
                 {64, 64, 3, false, true, -1}, {64, 64, 3, false, true, -1},
                 {64, 64, 2, true, false, 5},  {64, 64, 2, false, true, -1},
                 {64, 32, 1, true, false, 3},  {32, 32, 1, false, true, -1},
                 {32, 16, 0, true, false, 1},  {16, 16, 0, false, true, -1}};
  std::vector<UNetLayer> L;
  size_t off = 0;
  for (const D& e : d) {
    UNetLayer l;
    l.cin = e.cin; l.cout = e.cout; l.level = e.level; l.ups = e.ups; l.relu = e.relu;
    l.skip = e.skip;
    l.woff = off;
    off += (size_t)e.cout * 9 * e.cin;
    l.boff = off;
    off += e.cout;
    L.push_back(l);
  }
  return L;
}

int grid_for(size_t n, int sms) {
  size_t g = (n + 255) / 256;
  const size_t cap = (size_t)sms * 8;
  return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

// --- launch helpers (dispatch on the channel counts) -----------------------

template <int CIN, int COUT, bool UPS, bool MASK, bool ADD, bool RELU>
void conv_t(const ConvP& p, int sms, cudaStream_t s) {
  constexpr int smem = conv_smem<CIN, COUT>();
  auto k = k_conv<CIN, COUT, UPS, MASK, ADD, RELU>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  const int tiles = ((p.W + TW - 1) / TW) * ((p.H + TH - 1) / TH) * p.n;
  const int g = tiles < 2 * sms ? tiles : 2 * sms;
  k<<<g, NTH, smem, s>>>(p);
  note_launch();
}

// channel pairs of the upsampling decoder layers (64->64, 64->32, 32->16)
template <int CI, int CO>
constexpr bool up_pair() {
  return (CI == 64 && CO == 64) || (CI == 64 && CO == 32) || (CI == 32 && CO == 16);
}
// channel pairs of ReLU layers (encoder and decoder second convolutions)
template <int CI, int CO>
constexpr bool relu_pair() {
  return (CI == 16 && CO == 16) || (CI == 16 && CO == 32) || (CI == 32 && CO == 32) ||
         (CI == 32 && CO == 64) || (CI == 64 && CO == 64);
}

// forward layer: upsampling + skip add (decoder) or conv + ReLU
template <int CIN, int COUT>
void conv_fwd(const ConvP& p, bool ups, int sms, cudaStream_t s) {
  if constexpr (up_pair<CIN, COUT>()) {
    if (ups) {
      conv_t<CIN, COUT, true, false, true, false>(p, sms, s);
      return;
    }
  }
  if constexpr (relu_pair<CIN, COUT>()) conv_t<CIN, COUT, false, false, false, true>(p, sms, s);
}
// input gradient: conv of the output gradient (masked by the ReLU output
// for ReLU layers) with the flipped, transposed weights; CIN/COUT here are
// the layer's COUT/CIN
template <int CIN, int COUT>
void conv_bwd(const ConvP& p, bool mask, int sms, cudaStream_t s) {
  if constexpr (relu_pair<COUT, CIN>()) {
    if (mask) {
      conv_t<CIN, COUT, false, true, false, false>(p, sms, s);
      return;
    }
  }
  if constexpr (up_pair<COUT, CIN>()) conv_t<CIN, COUT, false, false, false, false>(p, sms, s);
}

void conv_mma(int cin, int cout, const ConvP& p, bool ups, bool bwd, bool mask, int sms,
              cudaStream_t s) {
#define SCF_CONV(CI, CO)                           \
  if (cin == CI && cout == CO) {                   \
    if (bwd) conv_bwd<CI, CO>(p, mask, sms, s);    \
    else conv_fwd<CI, CO>(p, ups, sms, s);         \
    return;                                        \
  }
  SCF_CONV(16, 16) SCF_CONV(16, 32) SCF_CONV(32, 16) SCF_CONV(32, 32) SCF_CONV(32, 64)
  SCF_CONV(64, 32) SCF_CONV(64, 64)
#undef SCF_CONV
}

}  // namespace

// a layer's convolution on the selected engine (tcgen05 unless a test or a
// measurement asks for the mma.sync kernel); map: the input's tensor map
// (device) for TMA staging, or null
void conv_dispatch(int engine, int cin, int cout, const ConvP& p, bool ups, bool bwd, bool mask,
                   int sms, int* err, const CUtensorMap* map, cudaStream_t s) {
  if (engine == 1 || engine == 2)
    conv_tc(cin, cout, p, ups, bwd, mask, sms, err, engine == 1 ? map : nullptr, s);
  else conv_mma(cin, cout, p, ups, bwd, mask, sms, s);
}

namespace {

template <int CIN, int COUT, bool UPS, bool RELU>
void wgrad_t(const WgP& p, int sms, cudaStream_t s) {
  constexpr int smem = wgrad_smem<CIN, COUT>();
  auto k = k_wgrad<CIN, COUT, UPS, RELU>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  const int tiles = ((p.W + TW - 1) / TW) * ((p.H + TH - 1) / TH) * p.n;
  int g = (2 * sms + 8) / 9;
  if (g > tiles) g = tiles;
  k<<<dim3(g, 9), NTH, smem, s>>>(p);
  note_launch();
}

void wgrad_dispatch(int cin, int cout, const WgP& p, bool ups, bool relu, int sms,
                    cudaStream_t s) {
#define SCF_WG(CI, CO)                                                        \
  if (cin == CI && cout == CO) {                                              \
    if constexpr (up_pair<CI, CO>())                                          \
      if (ups) { wgrad_t<CI, CO, true, false>(p, sms, s); return; }           \
    if constexpr (relu_pair<CI, CO>())                                        \
      if (relu) { wgrad_t<CI, CO, false, true>(p, sms, s); return; }          \
    return;                                                                   \
  }
  SCF_WG(16, 16) SCF_WG(16, 32) SCF_WG(32, 16) SCF_WG(32, 32) SCF_WG(32, 64) SCF_WG(64, 32)
  SCF_WG(64, 64)
#undef SCF_WG
}

}  // namespace

const std::vector<UNetLayer>& UNet::layers() {
  static const std::vector<UNetLayer> L = make_layers();
  return L;
}

int UNet::num_params() {
  const auto& L = layers();
  return (int)(L.back().boff + L.back().cout) + 17;
}

int UNet::alloc(void** p, size_t bytes) {
  if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) return -1;
  allocs_.push_back(*p);
  cudaMemset(*p, 0, bytes ? bytes : 16);
  return 0;
}

int UNet::create(int n, int h, int w, bool train, int device) {
  if (n < 1 || h < 8 || w < 8 || h % 8 || w % 8) return -1;
  if (cudaSetDevice(device) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device);
  n_ = n; h_ = h; w_ = w; train_ = train;
  const int np = num_params();
  const auto& L = layers();
  if (alloc((void**)&params_, np * 4)) return -1;
  size_t nw = 0;
  for (const auto& l : L) nw += (size_t)l.cout * 9 * l.cin;
  if (alloc((void**)&wb_, nw * 2) || alloc((void**)&wt_, nw * 2)) return -1;
  const size_t p0 = (size_t)n * h * w;
  auto px = [&](int level) { return p0 >> (2 * level); };
  if (alloc((void**)&in_, p0 * 16 * 2) || alloc((void**)&z_, p0 * 4) ||
      alloc((void**)&red_, 4096 * 4) || alloc((void**)&tc_err_, 4))
    return -1;
  act_.assign(L.size(), nullptr);
  for (size_t i = 0; i < L.size(); ++i)
    if (alloc((void**)&act_[i], px(L[i].level) * L[i].cout * 2)) return -1;
  pool_.assign(3, nullptr);
  const int pc[3] = {16, 32, 64};
  for (int i = 0; i < 3; ++i)
    if (alloc((void**)&pool_[i], px(i + 1) * pc[i] * 2)) return -1;
  // tensor maps of the forward ReLU layers' inputs (TMA staging); a layer
  // whose map the driver does not accept stages its rows with its threads
  has_map_.assign(L.size(), 0);
  if (alloc((void**)&maps_, L.size() * sizeof(CUtensorMap))) return -1;
  {
    std::vector<CUtensorMap> hm(L.size());
    for (size_t i = 0; i < L.size(); ++i) {
      const void* in = i == 0 ? (const void*)in_
                       : (i == 2 || i == 4 || i == 6) ? (const void*)pool_[i / 2 - 1]
                                                      : (const void*)act_[i - 1];
      // an upsampling layer's input is the level below (half resolution)
      const int lv = L[i].level + (L[i].ups ? 1 : 0);
      has_map_[i] = conv_tma_map(&hm[i], in, n, h >> lv, w >> lv, L[i].cin) == 0;
    }
    if (cudaMemcpy(maps_, hm.data(), L.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice) !=
        cudaSuccess)
      return -1;
  }
  if (train) {
    if (alloc((void**)&grads_, np * 4) || alloc((void**)&m_, np * 4) || alloc((void**)&v_, np * 4) ||
        alloc((void**)&dz_, p0 * 4))
      return -1;
    // scratch gradients: four full-resolution buffers of 64 channels suffice
    g_.assign(4, nullptr);
    for (int i = 0; i < 4; ++i)
      if (alloc((void**)&g_[i], p0 * 64 * 2)) return -1;
  }
  cudaDeviceSynchronize();
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void UNet::destroy() {
  for (void* p : allocs_) cudaFree(p);
  allocs_.clear();
  act_.clear(); pool_.clear(); g_.clear();
  params_ = grads_ = m_ = v_ = z_ = dz_ = red_ = nullptr;
  tc_err_ = nullptr;
  maps_ = nullptr;
  has_map_.clear();
  wb_ = wt_ = in_ = nullptr;
}

void UNet::refresh_weights(cudaStream_t s) {
  size_t off = 0;
  for (const auto& l : layers()) {
    const int nw = l.cout * 9 * l.cin;
    k_weights<<<grid_for(nw, sms_), 256, 0, s>>>(params_ + l.woff, l.cin, l.cout, wb_ + off,
                                                 wt_ + off);
    note_launch();
    off += nw;
  }
}

int UNet::set_params_host(const float* p) {
  if (cudaMemcpy(params_, p, (size_t)num_params() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return -1;
  refresh_weights(0);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}

int UNet::get_params_host(float* p) {
  return cudaMemcpy(p, params_, (size_t)num_params() * 4, cudaMemcpyDeviceToHost) == cudaSuccess
             ? 0
             : -1;
}

void UNet::features(int i, int nx, int ny, int ld, const double* r, const double* cE,
                    const double* cN, const double* dg, float* sigma_out, cudaStream_t s) {
  float* sums = red_ + 2 * (i % 1024);
  cudaMemsetAsync(sums, 0, 8, s);
  k_feat_sums<<<grid_for((size_t)nx * ny, sms_), 256, 0, s>>>(nx, ny, ld, r, dg, sums);
  note_launch();
  k_features<<<grid_for((size_t)h_ * w_, sms_), 256, 0, s>>>(
      nx, ny, ld, r, cE, cN, dg, sums, sigma_out, in_ + (size_t)i * h_ * w_ * 16, h_, w_);
  note_launch();
}

void UNet::forward(cudaStream_t s) {
  const auto& L = layers();
  // inputs of each layer
  for (size_t i = 0; i < L.size(); ++i) {
    const UNetLayer& l = L[i];
    const int H = h_ >> l.level, W = w_ >> l.level;
    const bf16* in;
    if (i == 0) in = in_;
    else if (i == 2 || i == 4 || i == 6) {
      const int k = (int)i / 2 - 1;  // pool index 0,1,2
      const UNetLayer& src = L[i - 1];
      k_pool<<<grid_for((size_t)n_ * H * W * src.cout / 8, sms_), 256, 0, s>>>(
          act_[i - 1], pool_[k], n_, H * 2, W * 2, src.cout);
      note_launch();
      in = pool_[k];
    } else {
      in = act_[i - 1];
    }
    ConvP p{};
    p.in = in;
    p.bias = params_ + l.boff;
    p.add = l.skip >= 0 ? act_[l.skip] : nullptr;
    p.out = act_[i];
    p.n = n_; p.H = H; p.W = W;
    // BF16 weights are packed without the biases: offset = sum of previous W sizes
    size_t off = 0;
    for (size_t j = 0; j < i; ++j) off += (size_t)L[j].cout * 9 * L[j].cin;
    p.wt = wb_ + off;
    conv_dispatch(engine_, l.cin, l.cout, p, l.ups, false, false, sms_, tc_err_,
                  has_map_[i] ? maps_ + i : nullptr, s);
  }
  k_head<<<grid_for((size_t)n_ * h_ * w_, sms_), 256, 0, s>>>(
      act_.back(), params_ + num_params() - 17, (size_t)n_ * h_ * w_, z_);
  note_launch();
}

void UNet::correction(int nx, int ny, int pitch, const double* dg, const float* sigma, float* x,
                      cudaStream_t s) {
  k_correction<float><<<grid_for((size_t)nx * ny, sms_), 256, 0, s>>>(nx, ny, pitch, w_, dg,
                                                                      sigma, z_, x);
  note_launch();
}

// target of image i for training: t = e / sigma (FP32) and the mask dg > 0;
// e, dg in Fortran (nx, ny) order, the image h x w
__global__ void k_target(int nx, int ny, int H, int W, const double* __restrict__ e,
                         const double* __restrict__ dg, const float* __restrict__ sigma,
                         float* __restrict__ t, unsigned char* __restrict__ mask) {
  const float s = *sigma;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < (size_t)H * W;
       q += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(q % W), y = (int)(q / W);
    float v = 0.0f;
    unsigned char m = 0;
    if (x < nx && y < ny) {
      const size_t k = (size_t)y * nx + x;
      if (dg[k] > 0.0) {
        v = (float)e[k] / s;
        m = 1;
      }
    }
    t[q] = v;
    mask[q] = m;
  }
}

void UNet::target(int i, int nx, int ny, const double* e, const double* dg, const float* sigma,
                  float* t, unsigned char* mask, cudaStream_t s) {
  const size_t hw = (size_t)h_ * w_;
  k_target<<<grid_for(hw, sms_), 256, 0, s>>>(nx, ny, h_, w_, e, dg, sigma, t + i * hw,
                                             mask + i * hw);
  note_launch();
}

void UNet::loss(const float* t, const unsigned char* mask, float* loss_dev, cudaStream_t s) {
  const size_t hw = (size_t)h_ * w_;
  float* sums = red_ + 2048;
  cudaMemsetAsync(sums, 0, 2 * n_ * 4, s);
  const dim3 g((unsigned)((grid_for(hw, sms_) + n_ - 1) / n_ + 1), n_);
  k_loss_sums<<<g, 256, 0, s>>>(z_, t, mask, hw, sums);
  note_launch();
  k_loss_grad<<<g, 256, 0, s>>>(z_, t, mask, hw, sums, dz_);
  note_launch();
  k_loss_total<<<1, 1, 0, s>>>(sums, n_, loss_dev);
  note_launch();
}

void UNet::backward(cudaStream_t s) {
  const auto& L = layers();
  const int nl = (int)L.size();
  cudaMemsetAsync(grads_, 0, (size_t)num_params() * 4, s);
  std::vector<size_t> woff(nl);
  size_t off = 0;
  for (int j = 0; j < nl; ++j) { woff[j] = off; off += (size_t)L[j].cout * 9 * L[j].cin; }
  const size_t p0 = (size_t)n_ * h_ * w_;
  // head: gradient of d0 into g_[0]
  k_head_bwd<<<grid_for(p0, sms_), 256, 0, s>>>(act_.back(), params_ + num_params() - 17, dz_, p0,
                                                g_[0], grads_ + num_params() - 17);
  note_launch();
  // g_[0..2] rotate through the layer gradients.  The skip gradients of
  // e0, e1, e2 (outputs of layers 1, 3, 5), set by the decoder's add layers
  // 12, 10, 8, live in g_[3] until the encoder adds them to the gradient of
  // its pooled output: e2 (level 2, 64 ch) at 0, e1 (level 1, 32 ch) at
  // P2*64, e0 (level 0, 16 ch) after it.
  bf16* gskip[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  const size_t P1 = p0 / 4, P2 = p0 / 16;
  gskip[5] = g_[3];
  gskip[3] = g_[3] + P2 * 64;
  gskip[1] = g_[3] + P2 * 64 + P1 * 32;
  int a = 0;  // index of gcur in g_[0..2]
  auto other = [&](int x, int y) {
    for (int k = 0; k < 3; ++k)
      if (k != x && k != y) return k;
    return 0;
  };
  for (int i = nl - 1; i >= 0; --i) {
    const UNetLayer& l = L[i];
    const int H = h_ >> l.level, W = w_ >> l.level;
    // this layer's input tensor (forward)
    const bf16* xin;
    if (i == 0) xin = in_;
    else if (i == 2 || i == 4 || i == 6) xin = pool_[i / 2 - 1];
    else xin = act_[i - 1];
    // weight gradient
    WgP w{};
    w.dy = g_[a];
    w.y = l.relu ? act_[i] : nullptr;
    w.x = xin;
    w.dw = grads_ + l.woff;
    w.db = grads_ + l.boff;
    w.n = n_; w.H = H; w.W = W;
    wgrad_dispatch(l.cin, l.cout, w, l.ups, l.relu, sms_, s);
    if (l.skip >= 0) {
      // the add passes the gradient to the skip tensor unchanged
      cudaMemcpyAsync(gskip[l.skip], g_[a], (size_t)n_ * H * W * l.cout * 2,
                      cudaMemcpyDeviceToDevice, s);
    }
    if (i == 0) break;
    // input gradient (full resolution of this layer)
    const int b = other(a, -1);
    ConvP p{};
    p.in = g_[a];
    p.mask = l.relu ? act_[i] : nullptr;
    p.wt = wt_ + woff[i];
    p.bias = nullptr;
    p.out = g_[b];
    p.n = n_; p.H = H; p.W = W;
    conv_dispatch(engine_, l.cout, l.cin, p, false, true, l.relu, sms_, tc_err_, nullptr, s);
    int cur = b;
    if (l.ups) {  // gradient of nearest upsampling: 2x2 sums onto the coarse input
      const int c = other(a, b);
      k_sumpool<<<grid_for((size_t)n_ * H * W * l.cin / 32, sms_), 256, 0, s>>>(
          g_[b], g_[c], n_, H, W, l.cin);
      note_launch();
      cur = c;
    }
    if (i == 2 || i == 4 || i == 6) {
      // input was pool(e_{k}); e_k also feeds the decoder's skip add:
      // g(e_k) = gskip + 0.25 * up(g(pool))
      const UNetLayer& src = L[i - 1];
      const int c = other(cur, -1);
      k_unpool_add<<<grid_for((size_t)n_ * (H * 2) * (W * 2) * src.cout / 8, sms_), 256, 0, s>>>(
          gskip[i - 1], g_[cur], g_[c], n_, H * 2, W * 2, src.cout);
      note_launch();
      cur = c;
    }
    a = cur;
  }
}

void UNet::adam(float lr, float b1, float b2, float eps, int step, cudaStream_t s) {
  const int n = num_params();
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  k_adam<<<grid_for(n, sms_), 256, 0, s>>>(params_, grads_, m_, v_, n, lr, b1, b2, eps, c1, c2);
  note_launch();
  refresh_weights(s);
}

}  // namespace scf

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
struct scf_unet {
  scf::UNet net;
  cudaStream_t stream = nullptr;
  int device = 0;
  float* loss_dev = nullptr;
};

extern "C" {

int scf_unet_num_params(void) { return scf::UNet::num_params(); }

int scf_unet_create(scf_unet** out, int n, int h, int w, int device) {
  if (!out) return -1;
  *out = nullptr;
  scf_unet* u = new scf_unet();
  u->device = device;
  if (u->net.create(n, h, w, true, device) != 0 ||
      cudaMalloc((void**)&u->loss_dev, 4) != cudaSuccess) {
    delete u;
    return -2;
  }
  *out = u;
  return 0;
}

int scf_unet_destroy(scf_unet* u) {
  if (!u) return 0;
  cudaSetDevice(u->device);
  cudaDeviceSynchronize();
  if (u->loss_dev) cudaFree(u->loss_dev);
  delete u;
  return 0;
}

int scf_unet_set_stream(scf_unet* u, void* stream) {
  if (!u) return -1;
  u->stream = (cudaStream_t)stream;
  return 0;
}

int scf_unet_set_params(scf_unet* u, const float* p) {
  if (!u || !p) return -1;
  cudaSetDevice(u->device);
  return u->net.set_params_host(p) ? -2 : 0;
}

int scf_unet_get_params(scf_unet* u, float* p) {
  if (!u || !p) return -1;
  cudaSetDevice(u->device);
  cudaStreamSynchronize(u->stream);
  return u->net.get_params_host(p) ? -2 : 0;
}

int scf_unet_features(scf_unet* u, int i, int nx, int ny, const double* r, const double* cE,
                      const double* cN, const double* dg, float* sigma_out) {
  if (!u || i < 0 || i >= u->net.n_ || nx > u->net.w_ || ny > u->net.h_ || nx < 1 || ny < 1)
    return -1;
  cudaSetDevice(u->device);
  u->net.features(i, nx, ny, nx, r, cE, cN, dg, sigma_out, u->stream);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int scf_unet_target(scf_unet* u, int i, int nx, int ny, const double* e, const double* dg,
                    const float* sigma, float* t, unsigned char* mask) {
  if (!u || i < 0 || i >= u->net.n_ || nx > u->net.w_ || ny > u->net.h_ || !e || !dg || !sigma ||
      !t || !mask)
    return -1;
  cudaSetDevice(u->device);
  u->net.target(i, nx, ny, e, dg, sigma, t, mask, u->stream);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int scf_unet_set_input(scf_unet* u, const float* x) {
  if (!u || !x) return -1;
  cudaSetDevice(u->device);
  const size_t np = (size_t)u->net.n_ * u->net.h_ * u->net.w_;
  std::vector<__nv_bfloat16> h(np * 16);
  for (size_t q = 0; q < np; ++q)
    for (int c = 0; c < 16; ++c) h[q * 16 + c] = __float2bfloat16_rn(c < 5 ? x[q * 5 + c] : 0.0f);
  cudaStreamSynchronize(u->stream);
  return cudaMemcpy(u->net.in_, h.data(), h.size() * 2, cudaMemcpyHostToDevice) == cudaSuccess
             ? 0
             : -2;
}

// -3 when a tcgen05 convolution's bounded wait ran out since the last check
// (the flag is cleared); -2 for a CUDA error
static int tc_status(scf_unet* u) {
  int e = 0;
  if (cudaMemcpyAsync(&e, u->net.tc_err_, 4, cudaMemcpyDeviceToHost, u->stream) != cudaSuccess ||
      cudaStreamSynchronize(u->stream) != cudaSuccess)
    return -2;
  if (e) {
    cudaMemsetAsync(u->net.tc_err_, 0, 4, u->stream);
    cudaStreamSynchronize(u->stream);
    return -3;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int scf_unet_set_engine(scf_unet* u, int engine) {
  if (!u || engine < 0 || engine > 2) return -1;
  u->net.engine_ = engine;
  return 0;
}

int scf_unet_forward(scf_unet* u, float* z, int device) {
  if (!u) return -1;
  cudaSetDevice(u->device);
  u->net.forward(u->stream);
  if (z) {
    const size_t np = (size_t)u->net.n_ * u->net.h_ * u->net.w_;
    if (cudaMemcpyAsync(z, u->net.z_, np * 4,
                        device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                        u->stream) != cudaSuccess)
      return -2;
  }
  if (cudaStreamSynchronize(u->stream) != cudaSuccess) return -2;
  return tc_status(u);
}

int scf_unet_conv(int engine, int cin, int cout, int ups, int bwd, int mask, const void* in,
                  const void* maskp, const void* wt, const float* bias, const void* add,
                  void* out, int n, int H, int W, void* stream) {
  if (engine < 0 || engine > 2 || n < 1 || H < 1 || W < 1 || !in || !wt || !out ||
      (ups && (bwd || H % 2 || W % 2 || !add)) || (mask && (!bwd || !maskp)) ||
      (!bwd && !ups && !bias))
    return -1;
  scf::ConvArgs a{};
  a.in = (const __nv_bfloat16*)in;
  a.mask = (const __nv_bfloat16*)maskp;
  a.wt = (const __nv_bfloat16*)wt;
  a.bias = bias;
  a.add = (const __nv_bfloat16*)add;
  a.out = (__nv_bfloat16*)out;
  a.n = n; a.H = H; a.W = W;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaStream_t s = (cudaStream_t)stream;
  int* err = nullptr;
  if (cudaMalloc((void**)&err, 4) != cudaSuccess) return -2;
  cudaMemsetAsync(err, 0, 4, s);
  // forward layers on engine 1: the input's tensor map for TMA staging
  CUtensorMap* dmap = nullptr;
  if (engine == 1 && !bwd) {
    CUtensorMap hm;
    if (scf::conv_tma_map(&hm, in, n, ups ? H / 2 : H, ups ? W / 2 : W, cin) == 0 &&
        cudaMalloc((void**)&dmap, sizeof(CUtensorMap)) == cudaSuccess)
      cudaMemcpy(dmap, &hm, sizeof(CUtensorMap), cudaMemcpyHostToDevice);
  }
  scf::conv_dispatch(engine, cin, cout, a, ups != 0, bwd != 0, mask != 0, sms, err, dmap, s);
  int e = 0;
  int rc = (cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
            cudaStreamSynchronize(s) == cudaSuccess && cudaGetLastError() == cudaSuccess)
               ? 0
               : -2;
  cudaFree(err);
  if (dmap) cudaFree(dmap);
  if (rc == 0 && e) rc = -3;
  return rc;
}

int scf_unet_loss(scf_unet* u, const float* t, const unsigned char* mask, float* loss_out) {
  if (!u || !t || !mask) return -1;
  cudaSetDevice(u->device);
  u->net.loss(t, mask, u->loss_dev, u->stream);
  if (loss_out &&
      cudaMemcpyAsync(loss_out, u->loss_dev, 4, cudaMemcpyDeviceToHost, u->stream) != cudaSuccess)
    return -2;
  return cudaStreamSynchronize(u->stream) == cudaSuccess ? 0 : -2;
}

int scf_unet_set_dz(scf_unet* u, const float* dz) {
  if (!u || !dz) return -1;
  cudaSetDevice(u->device);
  const size_t np = (size_t)u->net.n_ * u->net.h_ * u->net.w_;
  cudaStreamSynchronize(u->stream);
  return cudaMemcpy(u->net.dz_, dz, np * 4, cudaMemcpyHostToDevice) == cudaSuccess ? 0 : -2;
}

int scf_unet_backward(scf_unet* u) {
  if (!u) return -1;
  cudaSetDevice(u->device);
  u->net.backward(u->stream);
  if (cudaStreamSynchronize(u->stream) != cudaSuccess) return -2;
  return tc_status(u);
}

int scf_unet_get_grads(scf_unet* u, float* g) {
  if (!u || !g) return -1;
  cudaSetDevice(u->device);
  cudaStreamSynchronize(u->stream);
  return cudaMemcpy(g, u->net.grads_, (size_t)scf::UNet::num_params() * 4,
                    cudaMemcpyDeviceToHost) == cudaSuccess
             ? 0
             : -2;
}

int scf_unet_adam(scf_unet* u, float lr, float b1, float b2, float eps, int step) {
  if (!u || step < 1) return -1;
  cudaSetDevice(u->device);
  u->net.adam(lr, b1, b2, eps, step, u->stream);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // extern "C"
