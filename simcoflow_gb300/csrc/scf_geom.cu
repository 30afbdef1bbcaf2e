// scf_geom.cu -- the cut-cell geometry of Grid_Preprocess on the GPU
// (src/Cutcell_Mod.f90:18-397): Cell_Geo_Cal for the pressure cells with
// Edge_Geo_Cal (:34-300, :302-337), the clamps of the U and V cells,
// DefineMomentumExchangeCell (:360-397) and NumberExternalCell (:340-358),
// from the solid level-set fields that Initial_Clsvof leaves in the cells.
//
// The reference runs these as loops over i (outer) and j (inner) that update
// arrays in place.  Every loop but one touches each element from one
// iteration only, so it runs as one thread per cell here.  The exception is
// the solid/degenerate-cell rule (:215-244): a cell whose apertures vanish in
// one direction becomes solid and zeroes the faces it shares with its four
// neighbours, and the test of cell (i,j) sees the faces already zeroed by
// cells (i-1,j) and (i,j-1) but not by (i+1,j), (i,j+1).  Its outcome is the
// unique solution of status(i,j) = solid(i,j) or degenerate(status(i-1,j),
// status(i,j-1)), monotone in the predecessors' statuses, which a few
// parallel fixed-point sweeps reach (one per link of the longest chain of
// consecutive degenerate cells; the host stops when a sweep changes
// nothing).  Arithmetic is IEEE FP64 in the reference's operation order, so
// the results are bit-identical to a CPU restatement.  NumberExternalCell
// numbers the kept cells with j fastest: counts per (column, row-group)
// strip, a scan over the strips, and a walk of each strip from its offset.
#include <cstdint>

#include "scf_internal.cuh"
#include "scf_geom_gpu.cuh"

namespace scf {
namespace {

constexpr double kEps = 1.0e-3, kEpsF = 1.0e-2, kRnd = 1.0e-24;
constexpr int kRG = 32;  // row groups of the numbering

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
// IEEE division, correctly rounded, on the integer pipe
__device__ __forceinline__ double dvd(double a, double b) { return div_rn(a, b); }

#define G1(a, i, j) (a)[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx]
#define G0(a, i, j) (a)[(size_t)(i) + (size_t)(j) * (size_t)(nx + 2)]

// l >= 1e-14 for a non-NaN double by its bit pattern (integer pipe; an FP64
// compare issues on GB300's slow FP64 pipe); NaN compares false as in IEEE
__device__ __forceinline__ bool ge_e14(double l) {
  const long long b = __double_as_longlong(l);
  return (b & 0x7fffffffffffffffll) <= 0x7ff0000000000000ll && b >= 0x3d06849b86a12b9bll;
}

// IEEE comparisons of a double with a constant c > 0 on the integer pipe:
// for non-NaN x the signed 64-bit bit patterns order like the values when c
// is positive (negative x, -0 included, have negative patterns); NaN compares
// false.  gt_neg(x, c) is x > -c.
__device__ __forceinline__ bool nan_b(long long b) {
  return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}
__device__ __forceinline__ bool gt(double x, double c) {
  const long long b = __double_as_longlong(x);
  return !nan_b(b) && b > __double_as_longlong(c);
}
__device__ __forceinline__ bool ge(double x, double c) {
  const long long b = __double_as_longlong(x);
  return !nan_b(b) && b >= __double_as_longlong(c);
}
__device__ __forceinline__ bool lt(double x, double c) {
  const long long b = __double_as_longlong(x);
  return !nan_b(b) && b < __double_as_longlong(c);
}
__device__ __forceinline__ bool gt_neg(double x, double c) {
  const long long b = __double_as_longlong(x);
  return !nan_b(b) && (b >= 0 || (b & 0x7fffffffffffffffll) < __double_as_longlong(c));
}

// Edge_Geo_Cal: solid fraction of the edge p1-p2 under the linear level set
__device__ __forceinline__ double edge_solid(double p1x, double p1y, double p2x, double p2y,
                                             double a, double b, double p) {
  const double l1 = add(add(mul(a, p1x), mul(b, p1y)), p);
  const double l2 = add(add(mul(a, p2x), mul(b, p2y)), p);
  const bool g1 = ge_e14(l1), g2 = ge_e14(l2);
  const bool n1 = !isnan(l1), n2 = !isnan(l2);
  if (g1 && g2) return 0.0;
  if (!g1 && n1 && !g2 && n2) return 1.0;
  if (g1 && !g2 && n2) return dvd(fabs(l2), add(fabs(l1), fabs(l2)));
  return dvd(fabs(l1), add(fabs(l1), fabs(l2)));
}

// apertures of every P cell from its solid level set, the wall length from
// the solid apertures, then the open apertures 1 - solid
__global__ void k_geo_faces(GeoIn in, GeoOut o) {
  pdl_wait();
  const int nx = in.nx, ny = in.ny;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny; iy += gridDim.y * 8) {
    const int i = ix + 1, j = iy + 1;
    const double dx = G1(in.dx, i, j), dy = G1(in.dy, i, j);
    const double a = G1(in.nxS, i, j), b = G1(in.nyS, i, j), p = G1(in.phiS, i, j);
    G1(o.vofS, i, j) = G1(in.vofS, i, j);
    G1(o.nxS, i, j) = a;
    G1(o.nyS, i, j) = b;
    // Far from the body every corner's level-set value is >= 1e-14 (deep
    // inside, < 1e-14): every edge gives exactly 0 (1), the wall length 0 and
    // the open apertures exactly 1 (0).  The test runs in FP32 on values
    // widened and narrowed by bit manipulation, with a margin far above FP32
    // rounding, so it only ever takes cells whose FP64 result is certain.
    const float pf = d2f_rn(p), af = fabsf(d2f_rn(a)), bf = fabsf(d2f_rn(b));
    const float reach = 0.5f * (af * d2f_rn(dx) + bf * d2f_rn(dy));
    const float margin = 1.0e-4f * (fabsf(pf) + reach) + 1.0e-12f;
    const bool out = pf - reach > margin, in_ = pf + reach < -margin;
    if (out || in_) {
      const double ap = out ? 1.0 : 0.0;
      G1(o.WlLh, i, j) = 0.0;
      G0(o.aW, i, j) = ap; G0(o.aE, i, j) = ap; G0(o.aN, i, j) = ap; G0(o.aS, i, j) = ap;
      continue;
    }
    const double x0 = mul(-dx, 0.5), x1 = mul(dx, 0.5), y0 = mul(-dy, 0.5), y1 = mul(dy, 0.5);
    const double w = edge_solid(x0, y0, x0, y1, a, b, p);
    const double n = edge_solid(x0, y1, x1, y1, a, b, p);
    const double e = edge_solid(x1, y1, x1, y0, a, b, p);
    const double s = edge_solid(x1, y0, x0, y0, a, b, p);
    const double tx = mul(sub(e, w), dx), ty = mul(sub(n, s), dy);
    G1(o.WlLh, i, j) = __dsqrt_rn(add(mul(tx, tx), mul(ty, ty)));
    G0(o.aW, i, j) = sub(1.0, w);
    G0(o.aE, i, j) = sub(1.0, e);
    G0(o.aN, i, j) = sub(1.0, n);
    G0(o.aS, i, j) = sub(1.0, s);
  }
}

// 2 a b / (a + b + 1e-24); two fully open (1, 1) or closed (0, 0) faces give
// exactly 1 or 0 (2 / (2 + 1e-24) rounds to 1), without the FP64 division
__device__ __forceinline__ double hmean(double a, double b) {
  const long long ba = __double_as_longlong(a), bb = __double_as_longlong(b);
  if (ba == bb && (ba == 0x3ff0000000000000ll || ba == 0)) return a;
  return dvd(mul(mul(2.0, a), b), add(add(a, b), kRnd));
}

// harmonic averaging of the interior shared faces (i in 2..nx-1, j in
// 2..ny-1); each face is read and written by one thread only
__global__ void k_geo_average(int nx, int ny, GeoOut o) {
  pdl_wait();
  const int ix = blockIdx.x * 32 + threadIdx.x;
  const int i = ix + 2;
  if (i > nx - 1) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy + 2 <= ny - 1; iy += gridDim.y * 8) {
    const int j = iy + 2;
    G0(o.aN, i, j) = G0(o.aS, i, j + 1) = hmean(G0(o.aN, i, j), G0(o.aS, i, j + 1));
    const double av = hmean(G0(o.aE, i, j), G0(o.aW, i + 1, j));
    G0(o.aE, i, j) = av;
    G0(o.aW, i + 1, j) = av;
  }
}

// one fixed-point sweep of the solid/degenerate rule: st (0:nx+1,0:ny+1,
// ghosts 0) in, sn out; *changed set when a status turns on
__global__ void k_geo_status(int nx, int ny, GeoOut o, const uint8_t* st, uint8_t* sn,
                             int* changed) {
  pdl_wait();
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny; iy += gridDim.y * 8) {
    const int i = ix + 1, j = iy + 1;
    const double vs = G1(o.vofS, i, j);
    uint8_t s = G0(st, i, j);
    if (!s && lt(vs, 1.0 - kEps)) {
      const double w = G0(st, i - 1, j) ? 0.0 : G0(o.aW, i, j);
      const double so = G0(st, i, j - 1) ? 0.0 : G0(o.aS, i, j);
      if (lt(add(w, G0(o.aE, i, j)), kRnd) || lt(add(so, G0(o.aN, i, j)), kRnd)) {
        s = 1;
        *changed = 1;
      }
    }
    G0(sn, i, j) = s;
  }
}

__global__ void k_geo_status_init(int nx, int ny, GeoOut o, uint8_t* st) {
  pdl_wait();
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny; iy += gridDim.y * 8)
    G0(st, ix + 1, iy + 1) = gt(G1(o.vofS, ix + 1, iy + 1), 1.0 - kEps) ? 1 : 0;
}

// the rule's result: faces of a cell with status zero, and the faces its
// neighbours share with it; VofS = 1; then the wall length of solid cells
__global__ void k_geo_apply(int nx, int ny, GeoOut o, const uint8_t* st) {
  pdl_wait();
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny; iy += gridDim.y * 8) {
    const int i = ix + 1, j = iy + 1;
    const bool s = G0(st, i, j) != 0;
    double w = G0(o.aW, i, j), e = G0(o.aE, i, j), n = G0(o.aN, i, j), so = G0(o.aS, i, j);
    if (s || G0(st, i - 1, j)) w = 0.0;
    if (s || G0(st, i + 1, j)) e = 0.0;
    if (s || G0(st, i, j + 1)) n = 0.0;
    if (s || G0(st, i, j - 1)) so = 0.0;
    // ghost faces zeroed by boundary cells stay zero (they start at zero)
    G0(o.aW, i, j) = w; G0(o.aE, i, j) = e; G0(o.aN, i, j) = n; G0(o.aS, i, j) = so;
    double vs = G1(o.vofS, i, j);
    if (s) vs = 1.0;
    G1(o.vofS, i, j) = vs;
    if (__double_as_longlong(vs) == 0x3ff0000000000000ll) {  // |vs - 1| < 1e-24
      const double dx = G1(o.dx, i, j), dy = G1(o.dy, i, j);
      if (w == 0.0 || e == 0.0) G1(o.WlLh, i, j) = dy;
      if (n == 0.0 || so == 0.0) G1(o.WlLh, i, j) = dx;
    }
  }
}

// ICorProb corner rule (j in 1..ny-4), on the final VofS
__global__ void k_geo_corner(int nx, int ny, GeoOut o) {
  pdl_wait();
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy + 1 <= ny - 4; iy += gridDim.y * 8) {
    const int i = ix + 1, j = iy + 1;
    const double v0 = G1(o.vofS, i, j);
    if (!(gt_neg(v0, kEps) && lt(v0, kEps))) continue;
    const double v1 = G1(o.vofS, i, j + 1), v2 = G1(o.vofS, i, j + 2);
    const double dx = G1(o.dx, i, j);
    if (gt(v1, 0.6 - kEps) && lt(v1, 0.6 + kEps) && gt(v2, 0.6 - kEps) && lt(v2, 0.6 + kEps)) {
      G0(o.aN, i, j) = 0.40;
      G0(o.aS, i, j + 1) = 0.4;
      G1(o.WlLh, i, j) = mul(0.6, dx);
      G1(o.nyS, i, j) = -1.0;
      G1(o.nxS, i, j) = 0.0;
    }
    if (gt(v1, 1.0 - kEps) && lt(v1, 1.0 + kEps)) {
      G1(o.WlLh, i, j) = dx;
      G1(o.nyS, i, j) = -1.0;
      G1(o.nxS, i, j) = 0.0;
    }
  }
}

// U/V clamps and DefineMomentumExchangeCell; each thread reads and writes
// only its own cell's east/north faces and its neighbours' west/south ones
__global__ void k_geo_moex(GeoIn in, GeoOut o) {
  pdl_wait();
  const int nx = in.nx, ny = in.ny;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny; iy += gridDim.y * 8) {
    const int i = ix + 1, j = iy + 1;
    double vu = G1(in.vofS_u, i, j), vv = G1(in.vofS_v, i, j);
    if (gt(vu, 1.0 - kEps)) vu = 1.0;
    if (gt(vv, 1.0 - kEps)) vv = 1.0;
    G1(o.vofS_u, i, j) = vu;
    G1(o.vofS_v, i, j) = vv;
    int mu = 0, mv = 0;
    const double vs = G1(o.vofS, i, j);
    if (ge(vu, kEps) && lt(vu, 1.0 - kEps)) {
      if (i < nx) {
        if (ge(vs, 1.0 - kEps) || ge(G1(o.vofS, i + 1, j), 1.0 - kEps) || lt(G0(o.aE, i, j), kEpsF)) {
          mu = 1;
          G0(o.aE, i, j) = 0.0;
          G0(o.aW, i + 1, j) = 0.0;
        }
      } else if (ge(vs, 1.0 - kEps)) {
        mu = 1;
      }
    }
    if (ge(vv, kEps) && lt(vv, 1.0 - kEps)) {
      if (j < ny) {
        if (ge(vs, 1.0 - kEps) || ge(G1(o.vofS, i, j + 1), 1.0 - kEps) || lt(G0(o.aN, i, j), kEpsF)) {
          mv = 1;
          G0(o.aN, i, j) = 0.0;
          G0(o.aS, i, j + 1) = 0.0;
        }
      } else if (ge(vs, 1.0 - kEps)) {
        mv = 1;
      }
    }
    G1(o.moex_u, i, j) = mu;
    G1(o.moex_v, i, j) = mv;
  }
}

// NumberExternalCell, three families at once.  keep(f,i,j): P: VofS < 1-eps
// (i<=nx, j<=ny); U: i <= nx-1; V: j <= ny-1.
__device__ __forceinline__ bool keep(const GeoOut& o, int nx, int ny, int f, int i, int j) {
  if (f == 0) return lt(G1(o.vofS, i, j), 1.0 - kEps);
  if (f == 1) return i <= nx - 1 && lt(G1(o.vofS_u, i, j), 1.0 - kEps);
  return j <= ny - 1 && lt(G1(o.vofS_v, i, j), 1.0 - kEps);
}

// counts[f*(nx*kRG+1) + (i-1)*kRG + g]: kept cells of column i in row group
// g (rows g*rl+1 .. (g+1)*rl); one thread per (column, group), consecutive
// threads on consecutive columns (coalesced loads)
__global__ void k_geo_count(int nx, int ny, GeoOut o, int* counts) {
  pdl_wait();
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int g = blockIdx.y * 8 + threadIdx.y, f = blockIdx.z;
  if (i > nx || g >= kRG) return;
  const int rl = (ny + kRG - 1) / kRG, j0 = g * rl + 1, j1 = min(ny, j0 + rl - 1);
  int c = 0;
  for (int j = j0; j <= j1; ++j) c += keep(o, nx, ny, f, i, j) ? 1 : 0;
  counts[f * (nx * kRG + 1) + (i - 1) * kRG + g] = c;
}

// exclusive scan of each family's counts in (column, group) order: one block
// of 1024 threads per family walks the counts in tiles of 1024 (coalesced),
// scanning each tile by warp shuffles and carrying the running total
__global__ void k_geo_scan(int nx, int* counts) {
  pdl_wait();
  __shared__ int wsum[32];
  __shared__ int carry;
  const int n = nx * kRG;
  int* c = counts + blockIdx.x * (n + 1);
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int k = base + t;
    const int v = k < n ? c[k] : 0;
    int x = v;  // inclusive warp scan
    for (int s = 1; s < 32; s <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, s);
      if (lane >= s) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {  // scan of the 32 warp sums
      int z = wsum[lane];
      for (int s = 1; s < 32; s <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, z, s);
        if (lane >= s) z += y;
      }
      wsum[lane] = z;
    }
    __syncthreads();
    const int before = carry + (w > 0 ? wsum[w - 1] : 0) + x - v;
    if (k < n) c[k] = before;
    __syncthreads();
    if (t == 1023) carry = before + v;
    __syncthreads();
  }
  if (t == 0) c[n] = carry;  // total
}

// numbering with j fastest: each (column, group) thread walks its rows from
// its offset
__global__ void k_geo_number(int nx, int ny, GeoOut o, const int* counts) {
  pdl_wait();
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int g = blockIdx.y * 8 + threadIdx.y, f = blockIdx.z;
  if (i > nx || g >= kRG) return;
  int32_t* pn = f == 0 ? o.posnu_p : f == 1 ? o.posnu_u : o.posnu_v;
  const int rl = (ny + kRG - 1) / kRG, j0 = g * rl + 1, j1 = min(ny, j0 + rl - 1);
  int k = counts[f * (nx * kRG + 1) + (i - 1) * kRG + g];
  for (int j = j0; j <= j1; ++j) G0(pn, i, j) = keep(o, nx, ny, f, i, j) ? k++ : -1;
}

#undef G1
#undef G0

dim3 cell_grid(int nx, int ny) {
  const int gx = (nx + 31) / 32, gy0 = (ny + 7) / 8, cap = (152 * 16 + gx - 1) / gx;
  return dim3(gx, gy0 < cap ? gy0 : (cap < 1 ? 1 : cap));
}

}  // namespace

// The whole pipeline on stream s.  st0/st1: status buffers ((nx+2)(ny+2)
// bytes), counts: geometry_count_ints(nx) ints, flag: one device int,
// flag_host: pinned.
// Returns the number of fixed-point sweeps, or -1 if they did not settle
// within nx+ny+2 sweeps (not possible for a chain of finite length) or a
// CUDA call failed.
size_t geometry_count_ints(int nx) { return 3 * ((size_t)nx * kRG + 1); }

int geometry_build(const GeoIn& in, const GeoOut& o, uint8_t* st0, uint8_t* st1, int* counts,
                   int* flag, int* flag_host, int icorprob, cudaStream_t s) {
  const int nx = in.nx, ny = in.ny;
  const size_t n0 = (size_t)(nx + 2) * (ny + 2);
  const dim3 g = cell_grid(nx, ny), b(32, 8);
  // ghost faces and statuses start at zero, Posnu at -1
  cudaMemsetAsync(o.aE, 0, n0 * 8, s);
  cudaMemsetAsync(o.aW, 0, n0 * 8, s);
  cudaMemsetAsync(o.aN, 0, n0 * 8, s);
  cudaMemsetAsync(o.aS, 0, n0 * 8, s);
  cudaMemsetAsync(st0, 0, n0, s);
  cudaMemsetAsync(st1, 0, n0, s);
  cudaMemsetAsync(o.posnu_p, 0xff, n0 * 4, s);
  cudaMemsetAsync(o.posnu_u, 0xff, n0 * 4, s);
  cudaMemsetAsync(o.posnu_v, 0xff, n0 * 4, s);
  launch_k(k_geo_faces, g, b, 0, s, in, o);
  if (nx >= 3 && ny >= 3) launch_k(k_geo_average, cell_grid(nx - 2, ny - 2), b, 0, s, nx, ny, o);
  launch_k(k_geo_status_init, g, b, 0, s, nx, ny, o, st0);
  uint8_t *cur = st0, *nxt = st1;
  int sweeps = 0;
  for (;;) {
    cudaMemsetAsync(flag, 0, sizeof(int), s);
    launch_k(k_geo_status, g, b, 0, s, nx, ny, o, (const uint8_t*)cur, nxt, flag);
    cudaMemcpyAsync(flag_host, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    ++sweeps;
    uint8_t* t = cur; cur = nxt; nxt = t;
    if (!*flag_host) break;
    if (sweeps > nx + ny + 2) return -1;
  }
  launch_k(k_geo_apply, g, b, 0, s, nx, ny, o, (const uint8_t*)cur);
  if (icorprob && ny >= 5) launch_k(k_geo_corner, g, b, 0, s, nx, ny, o);
  launch_k(k_geo_moex, g, b, 0, s, in, o);
  const dim3 ng((nx + 31) / 32, kRG / 8, 3);
  launch_k(k_geo_count, ng, b, 0, s, nx, ny, o, counts);
  launch_k(k_geo_scan, dim3(3), dim3(1024), 0, s, nx, counts);
  launch_k(k_geo_number, ng, b, 0, s, nx, ny, o, (const int*)counts);
  if (cudaGetLastError() != cudaSuccess) return -1;
  return sweeps;
}

}  // namespace scf
