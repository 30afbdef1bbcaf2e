// scf_out.cu -- result files formatted on the GPU (include/scf_out.h): the
// Tecplot files of Print_Result_Tecplot_PCent / _UCent / _VCent
// (src/PrintResult.f90:39-168) and the ParaView file of Print_Result_VTK_2D
// (:165-190, through src/VTR_mod.f90).
//
// The files hold three header records and then every variable as a block of
// nx*ny records "(f24.14)", i fastest.  One kernel launch turns all values of
// all variables into their 25 bytes (24 characters and the line end) at
// once: a CTA formats 256 consecutive values of one variable into shared
// memory and stores the 6400 bytes with consecutive threads on consecutive
// bytes.  The host then copies the text in 64 MiB chunks into two pinned
// buffers and writes chunk k while chunk k+1 is being copied.
//
// The decimal conversion is exact integer arithmetic: |x| = m 2^-k with m the
// 53-bit significand; m 10^14 (< 2^100) in 128 bits shifted right by k, with
// the dropped bits deciding the round-to-nearest-even increment, gives the
// value in units of 1e-14.  No floating-point operation touches the digits.
#include <fcntl.h>
#include <unistd.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/scf_out.h"
#include "../../include/scf_proj.h"
#include "scf_internal.cuh"

namespace scf {
namespace {

constexpr int kW = 24, kRec = 25;      // field width, bytes per record
constexpr int kFmtThreads = 256;       // values per CTA
constexpr unsigned long long kP14 = 100000000000000ull;  // 10^14

// F24.14 text of x into o[0..23]
__device__ __forceinline__ void fmt_f24_14(double x, char* o) {
  using u64 = unsigned long long;
  using u128 = unsigned __int128;
  const u64 u = (u64)__double_as_longlong(x);
  const bool neg = (u >> 63) != 0;
  const int e = (int)((u >> 52) & 0x7ff);
  const u64 mant = u & 0xfffffffffffffull;
  auto right = [&](const char* s, int n) {  // right-justified word
    for (int i = 0; i < kW - n; ++i) o[i] = ' ';
    for (int i = 0; i < n; ++i) o[kW - n + i] = s[i];
  };
  auto stars = [&]() {
    for (int i = 0; i < kW; ++i) o[i] = '*';
  };
  if (e == 0x7ff) {
    if (mant) right("NaN", 3);
    else if (neg) right("-Infinity", 9);
    else right("Infinity", 8);
    return;
  }
  u64 I = 0, F = 0;  // integer part and the 14 fractional digits
  if (e != 0) {      // zero and subnormals round to 0
    const u64 m = mant | (1ull << 52);
    const int k = 1075 - e;  // |x| = m 2^-k
    if (k <= 0) {            // |x| >= 2^52: wider than the field
      stars();
      return;
    }
    const u128 P = (u128)m * kP14;
    u128 q = 0;
    if (k < 128) {  // for k >= 128, P 2^-k < 2^-28 rounds to 0
      q = P >> k;
      const u128 rem = P & ((((u128)1) << k) - 1);
      const u128 half = ((u128)1) << (k - 1);
      if (rem > half || (rem == half && (q & 1))) q += 1;
    }
    I = k <= 52 ? (m >> k) : 0;
    u128 f = q - (u128)I * kP14;  // in [0, 10^14]
    if (f >= kP14) {
      I += 1;
      f -= kP14;
    }
    F = (u64)f;
  }
  if (I >= (neg ? 100000000ull : 1000000000ull)) {  // sign + digits + '.' + 14 > 24
    stars();
    return;
  }
  int p = kW - 1;
  for (int d = 0; d < 14; ++d) {
    o[p--] = (char)('0' + (int)(F % 10));
    F /= 10;
  }
  o[p--] = '.';
  do {
    o[p--] = (char)('0' + (int)(I % 10));
    I /= 10;
  } while (I);
  if (neg) o[p--] = '-';
  while (p >= 0) o[p--] = ' ';
}

// ---------------------------------------------------------------------------
// ParaView VTR file of Print_Result_VTK_2D (src/PrintResult.f90:165-190)
// ---------------------------------------------------------------------------
using u64 = unsigned long long;
using u128 = unsigned __int128;
constexpr int kEW = 15;            // characters of one value
constexpr int kItem = kEW + 1;     // a blank and the value
constexpr int kPerLine = 5;        // values per record
constexpr int kLine = kPerLine * kItem + 1;
constexpr int kVtrThreads = 320;   // 64 whole records per CTA

// 5^q in 128 bits, 0 <= q <= 55
__device__ __forceinline__ u128 pow5(int q) {
  u128 r = 1;
  while (q >= 27) {  // 5^27 < 2^63
    r *= 7450580596923828125ull;
    q -= 27;
  }
  u64 t = 1;
  for (int k = 0; k < q; ++k) t *= 5;
  return r * t;
}

// X = m 2^e2 10^q (an exact rational): T = floor(X), D = X rounded to the
// nearest integer, ties to even.  Callers keep X below 10^10.
__device__ void scaled(u64 m, int e2, int q, u64& T, u64& D) {
  if (q >= 0) {
    // P = m 5^q as hi:lo (up to 24 + 124 bits), X = P 2^(e2+q)
    const u128 f = pow5(q);
    const u128 a = (u128)m * (u64)f, b = (u128)m * (u64)(f >> 64);
    const u128 lo = a + (b << 64);
    const u64 hi = (u64)(b >> 64) + (lo < a ? 1 : 0);
    const int sh = e2 + q;
    if (sh >= 0) {
      T = D = (u64)(lo << sh);
      return;
    }
    const int s = -sh;
    auto bit = [&](int k) -> u64 {
      return k < 128 ? (u64)(lo >> k) & 1 : (hi >> (k - 128)) & 1;
    };
    auto low_nonzero = [&](int k) -> bool {  // any of bits 0..k-1 set
      if (k <= 0) return false;
      if (k < 128) return (lo & ((((u128)1) << k) - 1)) != 0;
      if (lo != 0) return true;
      return k > 128 && (hi & ((1ull << (k - 128)) - 1)) != 0;
    };
    T = s < 128 ? (u64)((lo >> s) | ((u128)hi << (128 - s))) : hi >> (s - 128);
    const bool up = bit(s - 1) && (low_nonzero(s - 1) || (T & 1));
    D = T + (up ? 1 : 0);
  } else {
    // X = (m 2^e2) / 10^r with m 2^e2 < 2^128 and 10^r < 2^104
    const int r = -q;
    u128 p10 = 1;
    for (int k = 0; k < r; ++k) p10 *= 10;
    const u128 N = (u128)m << e2;
    const u128 t = N / p10, rem = N - t * p10;
    T = (u64)t;
    const bool up = 2 * rem > p10 || (2 * rem == p10 && (T & 1));
    D = T + (up ? 1 : 0);
  }
}

// The 15 characters of REAL(4) x: the sign ('-' or a blank), then the
// correctly rounded 9 significant digits "d.ddddddddE+dd" of the exact value
// of real(x, kind=4); "NaN", "Infinity", "-Infinity" right-justified.
__device__ void fmt_e15_8(double x, char* o) {
  const float f = __double2float_rn(x);
  const unsigned u = __float_as_uint(f);
  const bool neg = (u >> 31) != 0;
  const int be = (int)((u >> 23) & 0xff);
  const unsigned mant = u & 0x7fffffu;
  if (be == 0xff) {
    const char* w = mant ? "NaN" : neg ? "-Infinity" : "Infinity";
    const int n = mant ? 3 : neg ? 9 : 8;
    for (int i = 0; i < kEW - n; ++i) o[i] = ' ';
    for (int i = 0; i < n; ++i) o[kEW - n + i] = w[i];
    return;
  }
  u64 D = 0;
  int E = 0;
  if (be != 0 || mant != 0) {
    const u64 m = be ? (mant | 0x800000u) : mant;
    const int e2 = be ? be - 150 : -149;          // |f| = m 2^e2
    const int b = (63 - __clzll((long long)m)) + e2;  // floor(log2 |f|)
    E = (b * 78913) >> 18;  // floor(b log10 2) (Ryu's log10Pow2), floor(log10|f|) or one less
    u64 T;
    scaled(m, e2, 8 - E, T, D);
    if (T >= 1000000000ull) {
      ++E;
      scaled(m, e2, 8 - E, T, D);
    }
    if (D >= 1000000000ull) {  // rounded up to 10^9
      D = 100000000ull;
      ++E;
    }
  }
  o[0] = neg ? '-' : ' ';
  for (int k = 10; k >= 3; --k) {
    o[k] = (char)('0' + (int)(D % 10));
    D /= 10;
  }
  o[2] = '.';
  o[1] = (char)('0' + (int)D);
  o[11] = 'E';
  o[12] = E < 0 ? '-' : '+';
  const int ae = E < 0 ? -E : E;
  o[13] = (char)('0' + ae / 10);
  o[14] = (char)('0' + ae % 10);
}

// how one value list of the file is read from the Fortran arrays
enum VSrc : int {
  V_X = 0,  // x(i,1) of an (nx,ny) array, i = 1..nx
  V_Y,      // y(1,j), j = 1..ny
  V_ZERO,   // the one Z coordinate
  V_11,     // a(i,j) of (nx,ny)
  V_00,     // a(i,j) of (0:nx+1,0:ny+1)
  V_VEL3,   // (a(i,j), b(i,j), 0) of (0:nx+1,0:ny+1), per point
};
constexpr int kMaxVB = 12;
struct VBlock {
  int src;
  const double *a, *b;
  long long n, off;  // values, byte offset of the list in the file
};
struct VBlocks {
  int nb, nx;
  long long cta0[kMaxVB + 1];  // first CTA of each list
  VBlock v[kMaxVB];
};

__device__ __forceinline__ double vtr_value(const VBlock& B, int nx, long long k) {
  switch (B.src) {
    case V_X: return B.a[k];
    case V_Y: return B.a[k * nx];
    case V_ZERO: return 0.0;
    case V_11: return B.a[k];
    case V_00: {
      const long long i = k % nx + 1, j = k / nx + 1;
      return B.a[i + j * (nx + 2)];
    }
    default: {
      const long long c = k / 3, comp = k - 3 * c;
      if (comp == 2) return 0.0;
      const long long i = c % nx + 1, j = c / nx + 1;
      return (comp == 0 ? B.a : B.b)[i + j * (nx + 2)];
    }
  }
}

// One CTA formats 320 consecutive values of one list (64 records of five)
// into shared memory and stores the bytes with consecutive threads on
// consecutive bytes.
__global__ void __launch_bounds__(kVtrThreads) k_format_vtr(VBlocks d, char* out) {
  __shared__ char txt[kVtrThreads / kPerLine * kLine];
  int bi = 0;
  while (bi + 1 < d.nb && (long long)blockIdx.x >= d.cta0[bi + 1]) ++bi;
  const VBlock& B = d.v[bi];
  const long long v0 = ((long long)blockIdx.x - d.cta0[bi]) * kVtrThreads;
  const int t = threadIdx.x;
  const long long k = v0 + t;
  if (k < B.n) {
    char* o = txt + (t / kPerLine) * kLine + (t % kPerLine) * kItem;
    o[0] = ' ';
    fmt_e15_8(vtr_value(B, d.nx, k), o + 1);
    if (t % kPerLine == kPerLine - 1 || k == B.n - 1) o[kItem] = '\n';
  }
  __syncthreads();
  const long long nv = B.n - v0 < kVtrThreads ? B.n - v0 : kVtrThreads;
  const long long cnt = nv * kItem + (nv + kPerLine - 1) / kPerLine;
  char* dst = out + B.off + v0 / kPerLine * kLine;
  for (long long c = t; c < cnt; c += kVtrThreads) dst[c] = txt[c];
}

// plain array of values (diagnostics)
__global__ void k_format_e15_8(const double* v, long long n, char* out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    char o[kEW];
    fmt_e15_8(v[k], o);
    for (int c = 0; c < kEW; ++c) out[k * kEW + c] = o[c];
  }
}

// how one variable of a file is read from the Fortran arrays
enum Src : int {
  S_11 = 0,   // a(i,j) of an (nx,ny) array
  S_00,       // a(i,j) of an (0:nx+1,0:ny+1) array
  S_UAVG,     // 0.5*(a(i-1,j)+a(i,j)), (0:nx+1,0:ny+1)
  S_VAVG,     // 0.5*(a(i,j-1)+a(i,j)), (0:nx+1,0:ny+1)
  S_VOFA,     // 1 - a(i,j) - b(i,j), both (nx,ny)
};
constexpr int kMaxVars = 16;
struct Block {
  int src;
  const double *a, *b;
};
struct Blocks {
  int nvar, nx, ny;
  Block v[kMaxVars];
};

__device__ __forceinline__ double value_of(const Block& B, int nx, int i, int j) {
  const size_t k1 = (size_t)(i - 1) + (size_t)(j - 1) * nx;
  const size_t k0 = (size_t)i + (size_t)j * (nx + 2);
  switch (B.src) {
    case S_11: return B.a[k1];
    case S_00: return B.a[k0];
    case S_UAVG: return __dmul_rn(0.5, __dadd_rn(B.a[k0 - 1], B.a[k0]));
    case S_VAVG: return __dmul_rn(0.5, __dadd_rn(B.a[k0 - (nx + 2)], B.a[k0]));
    default: return __dsub_rn(__dsub_rn(1.0, B.a[k1]), B.b[k1]);
  }
}

// blockIdx.y = variable, blockIdx.x = run of 256 values
__global__ void __launch_bounds__(kFmtThreads) k_format_blocks(Blocks d, char* out) {
  __shared__ char txt[kFmtThreads * kRec];
  const int nx = d.nx;
  const long long n = (long long)nx * d.ny;
  const int t = threadIdx.x;
  const long long v0 = (long long)blockIdx.x * kFmtThreads;
  const long long idx = v0 + t;
  if (idx < n) {
    const int i = (int)(idx % nx) + 1, j = (int)(idx / nx) + 1;
    fmt_f24_14(value_of(d.v[blockIdx.y], nx, i, j), txt + t * kRec);
    txt[t * kRec + kW] = '\n';
  }
  __syncthreads();
  const long long cnt = (n - v0 < kFmtThreads ? n - v0 : kFmtThreads) * kRec;
  char* dst = out + ((long long)blockIdx.y * n + v0) * kRec;
  for (int b = t; b < cnt; b += kFmtThreads) dst[b] = txt[b];
}

// plain array of values (diagnostics)
__global__ void k_format_plain(const double* v, long long n, char* out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    char o[kW];
    fmt_f24_14(v[k], o);
    for (int c = 0; c < kW; ++c) out[k * kW + c] = o[c];
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

#define CKO(call)                                                        \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) {                                             \
      if (getenv("SCF_DEBUG"))                                           \
        fprintf(stderr, "scf_out: %s: %s\n", #call, cudaGetErrorString(e_)); \
      return e_ == cudaErrorMemoryAllocation ? SCF_ERR_NOMEM : SCF_ERR_CUDA; \
    }                                                                    \
  } while (0)

// the header records of a file (list-directed character output starts each
// record with a blank; adjacent character items are not separated)
std::string header(int kind, int nx, int ny) {
  std::string h = " title = \"flow\"\n";
  if (kind == SCF_TECPLOT_PCELL)
    h += " variables =\"x\",\"y\",\"p\",\"u\",\"v\",\"phi\",\"vof\",\"phiS\",\"vofS\""
         ",\"vofA\",\"Mres\",\"FluxU\",\"FluxV\",\"nxS\",\"nyS\"\n";
  else if (kind == SCF_TECPLOT_UCELL)
    h += " variables =\"x\",\"y\",\"u\",\"phi\",\"vof\",\"phiS\",\"vofS\",\"vofA\"\n";
  else
    h += " variables =\"x\",\"y\",\"v\",\"phi\",\"vof\",\"phiS\",\"vofS\",\"vofA\"\n";
  // format(1x,'zone i=',i5,',k=',i5,',f=block')
  auto i5 = [](int v) {
    char b[16];
    if (v < 0 || v > 99999) return std::string("*****");
    snprintf(b, sizeof b, "%5d", v);
    return std::string(b);
  };
  h += " zone i=" + i5(nx) + ",k=" + i5(ny) + ",f=block\n";
  return h;
}

int nvars(int kind) { return kind == SCF_TECPLOT_PCELL ? 15 : 8; }

// Device copies of the input arrays (host mode) and the variable table.
struct Staged {
  Blocks d{};
  void* mem = nullptr;
  ~Staged() {
    if (mem) cudaFree(mem);
  }
};

int stage(int kind, int nx, int ny, const void* fields, int flags, cudaStream_t s, Staged& st) {
  const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2);
  const bool dev = (flags & SCF_OUT_DEVICE_PTRS) != 0;
  // the arrays and their element counts, in a fixed order per kind
  const double* arr[16];
  size_t cnt[16];
  int na = 0;
  auto add = [&](const double* p, size_t c) {
    arr[na] = p;
    cnt[na] = c;
    return na++;
  };
  int ix, iy, ip = -1, iu = -1, iv = -1, iphi, ivof, iphiS, ivofS, imres = -1, iflux = -1,
      inxS = -1, inyS = -1, ivel = -1;
  if (kind == SCF_TECPLOT_PCELL) {
    const scf_tecplot_pcell* f = static_cast<const scf_tecplot_pcell*>(fields);
    ix = add(f->x, n1); iy = add(f->y, n1); ip = add(f->p, n0); iu = add(f->u, n0);
    iv = add(f->v, n0); iphi = add(f->phi, n1); ivof = add(f->vof, n1);
    iphiS = add(f->phiS, n1); ivofS = add(f->vofS, n1); imres = add(f->mres, n1);
    iflux = add(f->flux, 2 * n0); inxS = add(f->nxS, n1); inyS = add(f->nyS, n1);
  } else {
    const scf_tecplot_vcell* f = static_cast<const scf_tecplot_vcell*>(fields);
    ix = add(f->x, n1); iy = add(f->y, n1); ivel = add(f->vel, n0); iphi = add(f->phi, n1);
    ivof = add(f->vof, n1); iphiS = add(f->phiS, n1); ivofS = add(f->vofS, n1);
  }
  for (int a = 0; a < na; ++a)
    if (!arr[a]) return SCF_ERR_ARG;
  const double* darr[16];
  if (dev) {
    for (int a = 0; a < na; ++a) darr[a] = arr[a];
  } else {
    size_t total = 0;
    for (int a = 0; a < na; ++a) total += cnt[a];
    CKO(cudaMalloc(&st.mem, total * 8));
    double* p = static_cast<double*>(st.mem);
    for (int a = 0; a < na; ++a) {
      CKO(cudaMemcpyAsync(p, arr[a], cnt[a] * 8, cudaMemcpyHostToDevice, s));
      darr[a] = p;
      p += cnt[a];
    }
  }
  Blocks& d = st.d;
  d.nx = nx;
  d.ny = ny;
  int k = 0;
  auto var = [&](int src, int a, int b = -1) {
    d.v[k].src = src;
    d.v[k].a = darr[a];
    d.v[k].b = b >= 0 ? darr[b] : nullptr;
    ++k;
  };
  var(S_11, ix);
  var(S_11, iy);
  if (kind == SCF_TECPLOT_PCELL) {
    var(S_00, ip);
    var(S_UAVG, iu);
    var(S_VAVG, iv);
  } else {
    var(S_00, ivel);
  }
  var(S_11, iphi);
  var(S_11, ivof);
  var(S_11, iphiS);
  var(S_11, ivofS);
  var(S_VOFA, ivof, ivofS);
  if (kind == SCF_TECPLOT_PCELL) {
    var(S_11, imres);
    // FluxP(i,j,1) and FluxP(i,j,2) of Flux_n1(0:nx+1,0:ny+1,2)
    d.v[k] = {S_00, darr[iflux], nullptr}; ++k;
    d.v[k] = {S_00, darr[iflux] + n0, nullptr}; ++k;
    var(S_11, inxS);
    var(S_11, inyS);
  }
  d.nvar = k;
  return SCF_OK;
}

int check_args(int kind, int nx, int ny, const void* fields) {
  if (kind < SCF_TECPLOT_PCELL || kind > SCF_TECPLOT_VCELL || nx < 1 || ny < 1 || !fields)
    return SCF_ERR_ARG;
  return SCF_OK;
}

// Format the body of a file into dev_text (nvar * nx * ny * 25 bytes).
int format_body(const Staged& st, char* dev_text, cudaStream_t s) {
  const long long n = (long long)st.d.nx * st.d.ny;
  const dim3 g((unsigned)((n + kFmtThreads - 1) / kFmtThreads), (unsigned)st.d.nvar);
  k_format_blocks<<<g, kFmtThreads, 0, s>>>(st.d, dev_text);
  note_launch();
  CKO(cudaGetLastError());
  return SCF_OK;
}

// Pinned staging buffers shared by every writer call of the process, made
// once: pinning host memory costs about as much as copying through it.
constexpr size_t kChunk = (size_t)16 << 20;
constexpr int kBufs = 8;
struct PinPool {
  std::mutex mu;  // one streaming call at a time
  char* buf[kBufs] = {};
  bool ready = false;
};
PinPool& pin_pool() {
  static PinPool p;
  return p;
}

// Copy `body` bytes of device text to a sink in 16 MiB chunks: chunk c goes
// to pinned buffer c % kBufs, and `nsink` threads run the sink on chunks
// c = t, t + nsink, ... (a memcpy into the caller's buffer: 4 threads; a
// pwrite into the file at the chunk's offset: 1 thread, since writes to one
// file serialise in the file system anyway) while later chunks are still
// being copied; a buffer takes a new chunk only after its sink has finished.
template <class Sink>
int stream_out(const char* dtext, size_t body, cudaStream_t s, int nsink, Sink sink) {
  PinPool& pp = pin_pool();
  std::lock_guard<std::mutex> lock(pp.mu);
  if (!pp.ready) {
    for (int b = 0; b < kBufs; ++b)
      if (cudaMallocHost(&pp.buf[b], kChunk) != cudaSuccess) {
        for (int k = 0; k < b; ++k) cudaFreeHost(pp.buf[k]);
        return SCF_ERR_NOMEM;
      }
    pp.ready = true;
  }
  const size_t nch = (body + kChunk - 1) / kChunk;
  cudaEvent_t ev[kBufs];
  for (int b = 0; b < kBufs; ++b)
    if (cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming) != cudaSuccess) {
      for (int k = 0; k < b; ++k) cudaEventDestroy(ev[k]);
      return SCF_ERR_CUDA;
    }
  std::mutex mu;
  std::condition_variable cv;
  size_t issued = 0;           // chunks whose copy has been enqueued
  std::vector<char> done(nch, 0);
  std::atomic<int> rc{SCF_OK};
  auto worker = [&](int t) {
    for (size_t c = t; c < nch; c += nsink) {
      {
        std::unique_lock<std::mutex> l(mu);
        cv.wait(l, [&] { return issued > c || rc.load() != SCF_OK; });
      }
      if (rc.load() != SCF_OK) break;
      const int b = (int)(c % kBufs);
      if (cudaEventSynchronize(ev[b]) != cudaSuccess) {
        rc = SCF_ERR_CUDA;
      } else {
        const size_t off = c * kChunk, len = body - off < kChunk ? body - off : kChunk;
        if (!sink(pp.buf[b], len, off)) rc = SCF_ERR_IO;
      }
      {
        std::lock_guard<std::mutex> l(mu);
        done[c] = 1;
      }
      cv.notify_all();
    }
    cv.notify_all();
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nsink; ++t) th.emplace_back(worker, t);
  for (size_t c = 0; c < nch && rc.load() == SCF_OK; ++c) {
    const int b = (int)(c % kBufs);
    if (c >= (size_t)kBufs) {  // the buffer's previous chunk must be out
      std::unique_lock<std::mutex> l(mu);
      cv.wait(l, [&] { return done[c - kBufs] || rc.load() != SCF_OK; });
      if (rc.load() != SCF_OK) break;
    }
    const size_t off = c * kChunk, len = body - off < kChunk ? body - off : kChunk;
    if (cudaMemcpyAsync(pp.buf[b], dtext + off, len, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaEventRecord(ev[b], s) != cudaSuccess)
      rc = SCF_ERR_CUDA;
    {
      std::lock_guard<std::mutex> l(mu);
      issued = c + 1;
    }
    cv.notify_all();
  }
  cv.notify_all();
  for (auto& x : th) x.join();
  cudaStreamSynchronize(s);
  for (int b = 0; b < kBufs; ++b) cudaEventDestroy(ev[b]);
  return rc.load();
}

// ---- ParaView VTR file: layout and rendering ----

// "(I6)" after trim(adjustl())
std::string i6(int v) {
  if (v < -99999 || v > 999999) return "******";
  return std::to_string(v);
}

// The file as literal records and value lists, with their byte offsets
// (src/VTR_mod.f90:79-379 as Print_Result_VTK_2D calls it).
struct VtrLayout {
  std::vector<std::pair<size_t, std::string>> lits;
  VBlocks d{};
  size_t total = 0;
  long long ctas = 0;
};

// arr: x, y, u, v, p, phi, phiS, vof, vofS (device pointers or nulls)
void vtr_layout(int nx, int ny, const double* const* arr, VtrLayout& L) {
  size_t off = 0;
  auto lit = [&](const std::string& t) {
    L.lits.emplace_back(off, t);
    off += t.size();
  };
  auto vals = [&](int src, const double* a, const double* b, long long n) {
    VBlock& B = L.d.v[L.d.nb++];
    B = {src, a, b, n, (long long)off};
    off += (size_t)n * kItem + (size_t)((n + kPerLine - 1) / kPerLine);
  };
  const long long n = (long long)nx * ny;
  const std::string ni = i6(nx), nj = i6(ny);
  L.d.nx = nx;
  lit("<VTKFile type=\"RectilinearGrid\" version=\"0.1\" format=\"ascii\">\n"
      " <RectilinearGrid WholeExtent=\"1 " + ni + " 1 " + nj + " 1 1 \">\n"
      "  <Piece Extent=\"1 " + ni + " 1 " + nj + " 1 1 \">\n"
      "   <Coordinates>\n");
  const char* axes[3] = {"X", "Y", "Z"};
  for (int a = 0; a < 3; ++a) {
    lit(std::string("    <DataArray type=\"Float32\" Name=\"") + axes[a] +
        "_COORDINATES\" NumberOfComponents=\"1\" format=\"ascii\">\n");
    if (a == 0) vals(V_X, arr[0], nullptr, nx);
    else if (a == 1) vals(V_Y, arr[1], nullptr, ny);
    else vals(V_ZERO, nullptr, nullptr, 1);
    lit("    </DataArray>\n");
  }
  lit("   </Coordinates>\n   <PointData>\n");
  const char* vn[3] = {"Velocity", "X_Velocity", "Y_Velocity"};
  for (int a = 0; a < 3; ++a) {
    lit(std::string("        <DataArray type=\"Float32\" Name=\"") + vn[a] +
        "\" NumberOfComponents=\"" + (a == 0 ? "3" : "1") + "\" format=\"ascii\">\n");
    if (a == 0) vals(V_VEL3, arr[2], arr[3], 3 * n);
    else vals(V_00, arr[a == 1 ? 2 : 3], nullptr, n);
    lit("        </DataArray>\n");
  }
  const char* sn[5] = {"Pressure", "Levelset", "SolidLvs", "Vof", "SolidVof"};
  for (int a = 0; a < 5; ++a) {
    lit(std::string("         <DataArray type=\"Float32\" Name=\"") + sn[a] +
        "\" NumberOfComponents=\"1\" format=\"ascii\">\n");
    vals(a == 0 ? V_00 : V_11, arr[4 + a], nullptr, n);
    lit("         </DataArray>\n");
  }
  lit("     </PointData>\n   </Piece>\n  </RectilinearGrid>\n</VTKFile>\n");
  L.total = off;
  L.d.cta0[0] = 0;
  for (int b = 0; b < L.d.nb; ++b)
    L.d.cta0[b + 1] = L.d.cta0[b] + (L.d.v[b].n + kVtrThreads - 1) / kVtrThreads;
  L.ctas = L.d.cta0[L.d.nb];
}

// Render the whole file on the device and hand it to `sink` in chunks
// (stream_out); *total receives its size.
template <class Sink>
int vtr_run(int nx, int ny, const scf_vtr_fields* f, int flags, int device, int nsink,
            size_t* total, Sink sink) {
  if (nx < 1 || ny < 1 || !f) return SCF_ERR_ARG;
  const double* arr[9] = {f->x, f->y, f->u, f->v, f->p, f->phi, f->phiS, f->vof, f->vofS};
  for (auto a : arr)
    if (!a) return SCF_ERR_ARG;
  CKO(cudaSetDevice(device));
  const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2);
  const size_t cnt[9] = {n1, n1, n0, n0, n0, n1, n1, n1, n1};
  cudaStream_t s = nullptr;
  CKO(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  void* mem = nullptr;
  char* text = nullptr;
  int rc = SCF_OK;
  const double* darr[9];
  do {
    if (flags & SCF_OUT_DEVICE_PTRS) {
      for (int a = 0; a < 9; ++a) darr[a] = arr[a];
    } else {
      size_t tot = 0;
      for (size_t c : cnt) tot += c;
      if (cudaMalloc(&mem, tot * 8) != cudaSuccess) {
        rc = SCF_ERR_NOMEM;
        break;
      }
      double* p = static_cast<double*>(mem);
      for (int a = 0; a < 9 && rc == SCF_OK; ++a) {
        if (cudaMemcpyAsync(p, arr[a], cnt[a] * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
          rc = SCF_ERR_CUDA;
        darr[a] = p;
        p += cnt[a];
      }
      if (rc) break;
    }
    VtrLayout L;
    vtr_layout(nx, ny, darr, L);
    *total = L.total;
    if (cudaMalloc(&text, L.total) != cudaSuccess) {
      rc = SCF_ERR_NOMEM;
      break;
    }
    for (auto& l : L.lits)
      if (cudaMemcpyAsync(text + l.first, l.second.data(), l.second.size(),
                          cudaMemcpyHostToDevice, s) != cudaSuccess)
        rc = SCF_ERR_CUDA;
    if (rc) break;
    k_format_vtr<<<(unsigned)L.ctas, kVtrThreads, 0, s>>>(L.d, text);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    rc = stream_out(text, L.total, s, nsink, sink);
  } while (false);
  cudaStreamSynchronize(s);
  if (text) cudaFree(text);
  if (mem) cudaFree(mem);
  cudaStreamDestroy(s);
  return rc;
}

}  // namespace
}  // namespace scf

using namespace scf;

extern "C" {

int64_t scf_tecplot_size(int kind, int nx, int ny) {
  if (check_args(kind, nx, ny, "") != SCF_OK) return -1;
  return (int64_t)header(kind, nx, ny).size() + (int64_t)nvars(kind) * nx * ny * kRec;
}

int scf_tecplot_text(int kind, int nx, int ny, const void* fields, int flags, char* buf,
                     int64_t cap, int64_t* len, int device) {
  int rc = check_args(kind, nx, ny, fields);
  if (rc) return rc;
  if (!buf || !len) return SCF_ERR_ARG;
  const std::string h = header(kind, nx, ny);
  const size_t body = (size_t)nvars(kind) * nx * ny * kRec;
  *len = (int64_t)(h.size() + body);
  if (cap < *len) return SCF_ERR_ARG;
  CKO(cudaSetDevice(device));
  cudaStream_t s = nullptr;
  CKO(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  Staged st;
  char* text = nullptr;
  rc = stage(kind, nx, ny, fields, flags, s, st);
  if (rc == SCF_OK && cudaMalloc(&text, body) != cudaSuccess) rc = SCF_ERR_NOMEM;
  if (rc == SCF_OK) rc = format_body(st, text, s);
  memcpy(buf, h.data(), h.size());
  char* dst = buf + h.size();
  if (rc == SCF_OK)
    rc = stream_out(text, body, s, 4, [dst](const char* src, size_t n, size_t off) {
      memcpy(dst + off, src, n);
      return true;
    });
  cudaStreamSynchronize(s);
  if (text) cudaFree(text);
  cudaStreamDestroy(s);
  return rc;
}

int scf_tecplot_write(int kind, int nx, int ny, const void* fields, int flags, int64_t iter,
                      const char* dir, int device, double* ms) {
  int rc = check_args(kind, nx, ny, fields);
  if (rc) return rc;
  if (!dir) return SCF_ERR_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  // dir//'Tecplot/'//name//'_'//i8.8(iter)//'.dat'
  char num[16];
  if (iter < 0 || iter > 99999999) snprintf(num, sizeof num, "********");
  else snprintf(num, sizeof num, "%08lld", (long long)iter);
  static const char* names[3] = {"Pressure_", "Uvelocity_", "Vvelocity_"};
  std::string d(dir);
  while (!d.empty() && d.front() == ' ') d.erase(d.begin());  // trim(adjustl(dir))
  while (!d.empty() && d.back() == ' ') d.pop_back();
  const std::string path = d + "Tecplot/" + names[kind] + num + ".dat";
  const int fd = open(path.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) return SCF_ERR_IO;
  const std::string h = header(kind, nx, ny);
  const size_t body = (size_t)nvars(kind) * nx * ny * kRec;
  cudaStream_t s = nullptr;
  Staged st;
  char* text = nullptr;
  do {
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if ((rc = stage(kind, nx, ny, fields, flags, s, st))) break;
    if (cudaMalloc(&text, body) != cudaSuccess) {
      rc = SCF_ERR_NOMEM;
      break;
    }
    if ((rc = format_body(st, text, s))) break;
    if (pwrite(fd, h.data(), h.size(), 0) != (ssize_t)h.size()) {
      rc = SCF_ERR_IO;
      break;
    }
    const off_t base = (off_t)h.size();
    rc = stream_out(text, body, s, 1, [fd, base](const char* src, size_t n, size_t off) {
      size_t w = 0;
      while (w < n) {  // pwrite may write less than asked
        const ssize_t k = pwrite(fd, src + w, n - w, base + (off_t)(off + w));
        if (k <= 0) return false;
        w += (size_t)k;
      }
      return true;
    });
  } while (false);
  if (s) cudaStreamSynchronize(s);
  if (close(fd) != 0 && rc == SCF_OK) rc = SCF_ERR_IO;
  if (text) cudaFree(text);
  if (s) cudaStreamDestroy(s);
  if (ms)
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

int scf_tecplot_format(int kind, int nx, int ny, const void* fields, char* dev_text,
                       void* stream) {
  int rc = check_args(kind, nx, ny, fields);
  if (rc) return rc;
  if (!dev_text) return SCF_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Staged st;
  if ((rc = stage(kind, nx, ny, fields, SCF_OUT_DEVICE_PTRS, s, st))) return rc;
  return format_body(st, dev_text, s);
}

int64_t scf_vtr_size(int nx, int ny) {
  if (nx < 1 || ny < 1) return -1;
  const double* arr[9] = {};
  VtrLayout L;
  vtr_layout(nx, ny, arr, L);
  return (int64_t)L.total;
}

int scf_vtr_text(int nx, int ny, const scf_vtr_fields* fields, int flags, char* buf, int64_t cap,
                 int64_t* len, int device) {
  if (!buf || !len) return SCF_ERR_ARG;
  const int64_t need = scf_vtr_size(nx, ny);
  if (need < 0 || !fields) return SCF_ERR_ARG;
  *len = need;
  if (cap < need) return SCF_ERR_ARG;
  size_t total = 0;
  return vtr_run(nx, ny, fields, flags, device, 4, &total,
                 [buf](const char* src, size_t n, size_t off) {
                   memcpy(buf + off, src, n);
                   return true;
                 });
}

int scf_vtr_write(int nx, int ny, const scf_vtr_fields* fields, int flags, int64_t iter,
                  const char* dir, int device, double* ms) {
  if (nx < 1 || ny < 1 || !fields || !dir) return SCF_ERR_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  // trim(adjustl(dir))//'Paraview/'//'FlowField'//'_'//i8.8(iter)//'.vtr'
  char num[16];
  if (iter < 0 || iter > 99999999) snprintf(num, sizeof num, "********");
  else snprintf(num, sizeof num, "%08lld", (long long)iter);
  std::string d(dir);
  while (!d.empty() && d.front() == ' ') d.erase(d.begin());
  while (!d.empty() && d.back() == ' ') d.pop_back();
  const std::string path = d + "Paraview/FlowField_" + num + ".vtr";
  const int fd = open(path.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) return SCF_ERR_IO;
  size_t total = 0;
  int rc = vtr_run(nx, ny, fields, flags, device, 1, &total,
                   [fd](const char* src, size_t n, size_t off) {
                     size_t w = 0;
                     while (w < n) {
                       const ssize_t k = pwrite(fd, src + w, n - w, (off_t)(off + w));
                       if (k <= 0) return false;
                       w += (size_t)k;
                     }
                     return true;
                   });
  if (close(fd) != 0 && rc == SCF_OK) rc = SCF_ERR_IO;
  if (ms)
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

int scf_format_e15_8(const double* v, int64_t n, char* out, int device) {
  if (n < 0 || (n > 0 && (!v || !out))) return SCF_ERR_ARG;
  if (n == 0) return SCF_OK;
  CKO(cudaSetDevice(device));
  double* dv = nullptr;
  char* dout = nullptr;
  int rc = SCF_OK;
  if (cudaMalloc(&dv, (size_t)n * 8) != cudaSuccess ||
      cudaMalloc(&dout, (size_t)n * kEW) != cudaSuccess)
    rc = SCF_ERR_NOMEM;
  if (rc == SCF_OK && cudaMemcpy(dv, v, (size_t)n * 8, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = SCF_ERR_CUDA;
  if (rc == SCF_OK) {
    k_format_e15_8<<<152 * 8, 256>>>(dv, (long long)n, dout);
    note_launch();
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(out, dout, (size_t)n * kEW, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = SCF_ERR_CUDA;
  }
  if (dv) cudaFree(dv);
  if (dout) cudaFree(dout);
  return rc;
}

int scf_format_f24_14(const double* v, int64_t n, char* out, int device) {
  if (n < 0 || (n > 0 && (!v || !out))) return SCF_ERR_ARG;
  if (n == 0) return SCF_OK;
  CKO(cudaSetDevice(device));
  double* dv = nullptr;
  char* dout = nullptr;
  int rc = SCF_OK;
  if (cudaMalloc(&dv, (size_t)n * 8) != cudaSuccess ||
      cudaMalloc(&dout, (size_t)n * kW) != cudaSuccess)
    rc = SCF_ERR_NOMEM;
  if (rc == SCF_OK && cudaMemcpy(dv, v, (size_t)n * 8, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = SCF_ERR_CUDA;
  if (rc == SCF_OK) {
    k_format_plain<<<152 * 8, 256>>>(dv, (long long)n, dout);
    note_launch();
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(out, dout, (size_t)n * kW, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = SCF_ERR_CUDA;
  }
  if (dv) cudaFree(dv);
  if (dout) cudaFree(dout);
  return rc;
}

}  // extern "C"
