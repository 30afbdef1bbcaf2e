// scf_proj.cu -- host side of libscf_proj.so: the C-ABI declared in
// include/scf_proj.h.  Owns the device memory, the multigrid hierarchy and
// the CUDA graph of the PCG loop.
//
// The PCG loop runs entirely on the device: one CUDA graph holds a
// conditional WHILE node whose body is two PCG iterations (the direction
// vector, and in the flexible mixed-precision variant also z, ping-pong
// between two buffers); the convergence test in the last kernel of each
// iteration clears the loop condition.  No host round trip happens between
// the right-hand side and the final correction.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/scf_proj.h"
#include "scf_geom_gpu.cuh"
#include "scf_mg.cuh"
#include "scf_unet.cuh"
#include "scf_mgpre.cuh"

using namespace scf;

using bf16 = __nv_bfloat16;
using MgD = MgView<double, double, double>;
using MgF = MgView<float, bf16, float>;

struct scf_proj {
  int nx = 0, ny = 0;
  scf_opts opts;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // host-pointer mode: the solve's input copies run here, beside the
  // operator setup still running on `stream`
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_done = nullptr;
  cudaEvent_t late_done = nullptr;  // the copies only the correction reads
  // mixed setup: each level's conversion to FP32/BF16 runs on `aux` as soon
  // as the level exists, beside the coarsening of the next levels
  cudaStream_t aux = nullptr;
  cudaEvent_t lev_ev[32] = {}, aux_done = nullptr;
  // host mode: set_geometry's U/V arrays (read by the correction only), copied
  // by the next solve on the copy stream while the PCG runs
  struct Late {
    void* dst;
    const void* src;
    size_t bytes;
  } late[6] = {};
  bool late_pending = false;
  bool devptrs = false;
  bool mixed = false;
  int tile = SCF_TILE_64X32;  // point-smoother sweep tile (scf_proj_set_tile)

  // FP64 multigrid levels (setup hierarchy; level 0 is the fine operator of
  // the PCG, its b is the PCG residual r and its x the FP64 z)
  std::vector<LevelView> lev;
  std::vector<double*> di64;  // FP64 inverse diagonals
  std::vector<double*> x2_64; // second iterate buffer of each FP64 level
  std::vector<float*> x2_32;  // second iterate buffer of each mixed level
  // mixed levels (FP32 state, BF16 couplings), built from lev at assemble
  std::vector<MgF> mix;
  float* r32 = nullptr;  // FP32 copy of the PCG residual (mixed)
  // device tensor maps of the TMA-staged sweep, kSweepMaps per mixed level
  // (tma[l]: the level uses it)
  std::vector<CUtensorMap*> dmaps;
  std::vector<char> tma;
  // single-CTA tail of the V-cycle: levels tail0 .. L-1 (tail0 = 0: none)
  int tail0 = 0;
  TailDesc<double, double> tail64{};
  TailDesc<float, bf16> tail32{};
  // line smoother: transposed copy of each level (cE and cN swapped), used
  // for the lines along y; allocated when the line smoother is selected
  bool line = false;
  bool line_alloc = false;
  int ltail0 = 0;  // first level of the single-CTA line tail (0: none)
  TailDesc<double, double> ltail64{};
  TailDesc<float, bf16> ltail32{};
  std::vector<MgD> t64;
  std::vector<MgF> t32;
  // FP64 line factors of the kernel levels: [level][0 natural, 1 transposed]
  std::vector<LineFactors<double>> lf64n, lf64t;
  unsigned* aspect_bits = nullptr;  // device: largest cell aspect ratio (float bits)
  // learned preconditioner (SCF_PRECOND_LEARNED): network and its residual scale
  UNet* net = nullptr;
  float* net_sigma = nullptr;
  float* cscale = nullptr;      // device, one BF16 scale per level
  unsigned* maxbits = nullptr;  // device, one per level
  std::vector<void*> allocs;
  // PCG vectors (padded layout)
  double *xsol = nullptr, *pA = nullptr, *pB = nullptr, *q = nullptr, *bvec = nullptr;
  // coarsest-level dense inverse
  double* Ainv = nullptr;
  int* cmap = nullptr;
  int* ncoarse = nullptr;
  // scalars and reduction partials
  Scalars* sc = nullptr;
  Scalars* sc_diag = nullptr;
  double* part = nullptr;
  Scalars* sc_host = nullptr;  // pinned

  // Fortran-layout device arrays (host mode: owned staging; device mode:
  // caller's pointers)
  FortranIn fin{};
  double *st_dx = nullptr, *st_dy = nullptr, *st_dxU = nullptr, *st_dyV = nullptr;
  double *st_vof = nullptr, *st_phi = nullptr, *st_vofS = nullptr, *st_nyS = nullptr,
         *st_WlLh = nullptr;
  double *st_aE = nullptr, *st_aW = nullptr, *st_aN = nullptr, *st_aS = nullptr;
  int32_t *st_pp = nullptr, *st_pu = nullptr, *st_pv = nullptr, *st_mu = nullptr,
          *st_mv = nullptr;
  double *st_vsu = nullptr, *st_vsv = nullptr, *st_DpU = nullptr, *st_DpV = nullptr;
  // GPU-computed geometry (scf_proj_set_solid): outputs, host-mode input
  // staging, fixed-point and numbering scratch; allocated on first use
  bool geo_alloc = false;
  double *g_aE = nullptr, *g_aW = nullptr, *g_aN = nullptr, *g_aS = nullptr;
  double *g_WlLh = nullptr, *g_vofS = nullptr, *g_nxS = nullptr, *g_nyS = nullptr,
         *g_vsu = nullptr, *g_vsv = nullptr;
  int32_t *g_pp = nullptr, *g_pu = nullptr, *g_pv = nullptr, *g_mu = nullptr, *g_mv = nullptr;
  double* g_in[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  uint8_t *g_st0 = nullptr, *g_st1 = nullptr;
  int *g_counts = nullptr, *g_flag = nullptr, *g_flag_host = nullptr;
  int geo_sweeps = 0;
  double *st_us = nullptr, *st_vs = nullptr, *st_Pp = nullptr, *st_p = nullptr, *st_u = nullptr,
         *st_v = nullptr, *st_mres = nullptr;

  bool have_grid = false, have_geom = false, assembled = false;

  // graph of the PCG loop
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graph_cond = false;              // true: conditional while-node graph
  cudaGraph_t body_graph = nullptr;
  cudaGraphExec_t body_exec = nullptr;  // fallback: body only, host-polled
  long long body_launches = 0;          // kernel nodes of one loop body (two iterations)
  long long body_runs = 0;              // host-polled body graph launches of this solve
  long long pending_launches = 0;       // launches of an assembly not yet reported

  cudaEvent_t ev[8];
};

namespace {

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      if (getenv("SCF_DEBUG"))                                                         \
        fprintf(stderr, "scf: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(e_), \
                __FILE__, __LINE__);                                                   \
      return e_ == cudaErrorMemoryAllocation ? SCF_ERR_NOMEM : SCF_ERR_CUDA;           \
    }                                                                                  \
  } while (0)

int dev_alloc(scf_proj* h, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? SCF_ERR_NOMEM : SCF_ERR_CUDA;
  h->allocs.push_back(*p);
  e = cudaMemsetAsync(*p, 0, bytes ? bytes : 16, h->stream);
  return e == cudaSuccess ? SCF_OK : SCF_ERR_CUDA;
}

// padded array for a level: (ny+3)*pitch elements, base at row 2
template <class T>
int level_array(scf_proj* h, int ny, int pitch, T** base) {
  void* p = nullptr;
  size_t n = (size_t)(ny + 3) * pitch;
  int rc = dev_alloc(h, &p, n * sizeof(T));
  if (rc) return rc;
  *base = reinterpret_cast<T*>(p) + 2 * (size_t)pitch;
  return SCF_OK;
}

void destroy_graph(scf_proj* h) {
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->graph) cudaGraphDestroy(h->graph);
  if (h->body_exec) cudaGraphExecDestroy(h->body_exec);
  if (h->body_graph) cudaGraphDestroy(h->body_graph);
  h->gexec = nullptr; h->graph = nullptr; h->body_exec = nullptr; h->body_graph = nullptr;
}

MgD view64(scf_proj* h, int l) {
  const LevelView& L = h->lev[l];
  MgD v{};
  v.nx = L.nx; v.ny = L.ny; v.pitch = L.pitch;
  v.cE = L.cE; v.cN = L.cN; v.dg = L.dg; v.di = h->di64[l];
  v.x = L.x; v.b = L.b; v.xin = nullptr; v.csp = nullptr;
  return v;
}

// the two iterate buffers of a level; buffer 0 is the one in the base view
double* buf64(scf_proj* h, int l, int i) { return i == 0 ? h->lev[l].x : h->x2_64[l]; }
float* buf32(scf_proj* h, int l, int i) { return i == 0 ? h->mix[l].x : h->x2_32[l]; }

// the TMA-staged sweep runs on mixed levels of at least 128 x 64 cells whose
// tensor maps were accepted (SCF_NO_TMA turns it off)
bool tma_level(const scf_proj* h, int l) {
  static const bool off = getenv("SCF_NO_TMA") != nullptr;
  return !off && h->tile == SCF_TILE_64X32 && l < (int)h->tma.size() && h->tma[l];
}

// Largest level handled by the single-CTA tails (SCF_TAIL_CELLS overrides
// kTailMaxCells, for tuning; shared memory bounds it in any case).
long tail_cells() {
  static const long v = [] {
    const char* e = getenv("SCF_TAIL_CELLS");
    const long n = e ? atol(e) : 0;
    return n > 0 ? n : (long)kTailMaxCells;
  }();
  return v;
}

// The sweeps of one side of a V-cycle level as fused launches.  FP32
// levels: two red-black iterations per launch while two remain, then one
// (the second iteration reuses the tile staged by the first, halving the
// DRAM traffic; its extra halo work is cheap in FP32).  FP64 levels: one per
// launch -- the FP64 pipe, not DRAM, bounds them, and the wider halo would
// add FP64 work.
std::vector<int> sweep_launches(int n, bool fused2) {
  std::vector<int> c;
  for (; fused2 && n >= 2; n -= 2) c.push_back(2);
  for (; n > 0; --n) c.push_back(1);
  return c;
}

// Sweeps before (post: after) the coarse correction on level l: npre /
// npost, or the coarse schedule's count from level coarse_from down (point
// smoother: red-black iterations; line smoother: a step of x-lines then
// y-lines counts as two)
int sweeps_at(const scf_proj* h, int l, bool post) {
  const scf_opts& o = h->opts;
  return o.coarse_sweeps > 0 && l >= o.coarse_from ? o.coarse_sweeps : (post ? o.npost : o.npre);
}

// Buffer holding a level's result after its part of the V-cycle: sweep
// launches alternate buffers (down, then up, starting from buffer 0), the
// tail and the coarse solve write buffer 0.
int final_buf(scf_proj* h, int l) {
  if (h->line) return 0;  // line passes update in place
  const int L = (int)h->lev.size();
  const int lk = h->tail0 > 0 ? h->tail0 : L - 1;
  if (L == 1 || l >= lk) return 0;
  const int npre = (int)sweep_launches(sweeps_at(h, l, false), h->mixed).size();
  const int npost = (int)sweep_launches(sweeps_at(h, l, true), h->mixed).size();
  return (npre - 1 + npost) % 2;
}

// Enqueue one V-cycle.  `view(l)` is the base view of level l (level 0's b
// is the PCG residual), `buf(l, i)` its two iterate buffers.  do_rz: the
// last kernel reduces r.z and sets the PCG beta.
template <class T, class CT, class ViewFn, class BufFn>
void enqueue_vcycle_t(scf_proj* h, ViewFn view, BufFn buf, const TailDesc<T, CT>& tail,
                      Scalars* sc, bool do_rz, int flexible, cudaStream_t s) {
  using V = MgView<T, CT, T>;
  const int L = (int)h->lev.size();
  const bool fused2 = std::is_same<T, float>::value;
  const double om = h->opts.omega;
  if (L == 1) {
    V c = view(0);
    c.x = buf(0, 0);
    launch_coarse_solve_t(c, h->Ainv, h->cmap, h->ncoarse, sc, s);
    if (do_rz) launch_dot_rz_t<T, T>(c.nx, c.ny, c.pitch, c.b, c.x, flexible, sc, h->part, s);
    return;
  }
  // levels 0 .. lk-1 run as kernels; the tail (or the coarse solve) covers lk .. L-1
  const int lk = h->tail0 > 0 ? h->tail0 : L - 1;
  auto coarse_result = [&](int l) {  // level l with x = its final buffer
    V c = view(l);
    c.x = buf(l, final_buf(h, l));
    return c;
  };
  for (int l = 0; l < lk; ++l) {
    V f = view(l);
    const V c = view(l + 1);  // restriction target (its b)
    const std::vector<int> pre = sweep_launches(sweeps_at(h, l, false), fused2);
    const int npre = (int)pre.size();
    for (int it = 0; it < npre; ++it) {
      f.xin = it > 0 ? buf(l, (it - 1) % 2) : nullptr;
      f.x = buf(l, it % 2);
      if constexpr (std::is_same<T, float>::value) {
        if (tma_level(h, l)) {
          launch_sweep_tma(f, c, h->dmaps[l], it > 0 ? (it - 1) % 2 : 0, 0, it == 0, false,
                           it == npre - 1, false, om, flexible, sc, h->part, s, pre[it]);
          continue;
        }
      }
      launch_sweep(f, c, 0, it == 0, false, it == npre - 1, false, om, flexible, sc, h->part, s,
                   pre[it], h->tile);
    }
  }
  if (h->tail0 > 0) {
    launch_tail(tail, sc, s);
  } else {
    V c = view(L - 1);
    c.x = buf(L - 1, 0);
    launch_coarse_solve_t(c, h->Ainv, h->cmap, h->ncoarse, sc, s);
  }
  for (int l = lk - 1; l >= 0; --l) {
    V f = view(l);
    const V c = coarse_result(l + 1);
    const int npre = (int)sweep_launches(sweeps_at(h, l, false), fused2).size();
    const std::vector<int> post = sweep_launches(sweeps_at(h, l, true), fused2);
    const int npost = (int)post.size();
    for (int it = 0; it < npost; ++it) {
      f.xin = buf(l, (npre - 1 + it) % 2);
      f.x = buf(l, (npre + it) % 2);
      const bool rz = l == 0 && do_rz && it == npost - 1;
      if constexpr (std::is_same<T, float>::value) {
        if (tma_level(h, l)) {
          launch_sweep_tma(f, c, h->dmaps[l], (npre - 1 + it) % 2, 1, false, it == 0, false, rz,
                           om, flexible, sc, h->part, s, post[it]);
          continue;
        }
      }
      launch_sweep(f, c, 1, false, it == 0, false, rz, om, flexible, sc, h->part, s, post[it],
                   h->tile);
    }
  }
}

// the coarse-level schedule of a tail whose first level is level l0 of the
// hierarchy (tail levels are numbered from 0)
constexpr int kNoCoarse = 1 << 20;
template <class D>
void set_tail_coarse(D& d, const scf_opts& o, int l0) {
  d.cfrom = o.coarse_sweeps > 0 ? (o.coarse_from > l0 ? o.coarse_from - l0 : 0) : kNoCoarse;
  d.cpre = d.cpost = o.coarse_sweeps;
}

// V-cycle with the alternating zebra line smoother.  A smoothing step is
// x-lines (even rows, odd rows), then y-lines (even columns, odd columns) on
// the transposed level; the post-smoothing steps run the same passes in
// reverse order, so the V-cycle stays symmetric.  A step counts as two
// sweeps of npre / npost.  x and b move to the transposed layout by tiled
// transposes (b once per level and V-cycle).  Every pass updates x in place.
template <class T, class CT, class ViewFn, class TViewFn>
void enqueue_vcycle_line_t(scf_proj* h, ViewFn view, TViewFn tview, const TailDesc<T, CT>& tail,
                           Scalars* sc, bool do_rz, int flexible, cudaStream_t s) {
  using V = MgView<T, CT, T>;
  const int L = (int)h->lev.size();
  // steps per level (a step counts as two sweeps)
  auto steps = [h](int l, bool post) { return (sweeps_at(h, l, post) + 1) / 2; };
  const double om = h->opts.omega;
  auto to_t = [&](const V& f, const V& ft) {
    launch_transpose<T>(f.x, f.nx, f.ny, f.pitch, ft.x, ft.pitch, sc, s);
  };
  auto from_t = [&](const V& f, const V& ft) {
    launch_transpose<T>(ft.x, ft.nx, ft.ny, ft.pitch, f.x, f.pitch, sc, s);
  };
  // one pass: factored on FP64 levels that have factors, else the full solve
  // (which can also reduce the PCG's r.z on its last pass)
  bool rz_done = false;
  auto pass = [&](int l, bool tr, int colour, bool zero, bool rz = false) {
    const V L = tr ? tview(l) : view(l);
    if constexpr (std::is_same<T, double>::value) {
      if (l < (int)h->lf64n.size()) {
        launch_line_solve<double, double>(L, tr ? h->lf64t[l] : h->lf64n[l], colour, zero, sc, s);
        return;
      }
    }
    launch_line(L, colour, zero, sc, s, rz, flexible, h->part);
    rz_done = rz_done || rz;
  };
  // One alternating step.  The iterate lives in one layout at a time: a
  // pre-smoothing step ends on the transposed copy (the restriction reads
  // it there) unless another step follows; a post-smoothing step starts on
  // the transposed copy (the prolongation wrote it there) when it is the
  // first, and always ends in the natural layout.
  auto step = [&](int l, bool post, bool zero, bool edge, bool rz = false) {
    const V f = view(l), ft = tview(l);
    if (!post) {
      pass(l, false, 0, zero);
      pass(l, false, 1, false);
      to_t(f, ft);
      pass(l, true, 0, false);
      pass(l, true, 1, false);
      if (!edge) from_t(f, ft);
    } else {
      if (!edge) to_t(f, ft);
      pass(l, true, 1, false);
      pass(l, true, 0, false);
      from_t(f, ft);
      pass(l, false, 1, false);
      pass(l, false, 0, false, rz);
    }
  };
  // levels 0 .. lk-1 run as kernels; the tail (or the coarse solve) covers lk .. L-1
  const int lk = h->ltail0 > 0 ? h->ltail0 : L - 1;
  for (int l = 0; l < lk; ++l) {
    const V f = view(l), ft = tview(l);
    // level 0 gets b from the PCG; coarser levels get both layouts from the
    // restriction
    if (l == 0) launch_transpose<T>(f.b, f.nx, f.ny, f.pitch, ft.b, ft.pitch, sc, s);
    const int npre = steps(l, false);
    for (int it = 0; it < npre; ++it) step(l, false, it == 0, it == npre - 1);
    launch_resid_restrict_lt(ft, view(l + 1), tview(l + 1), sc, s);
  }
  if (h->ltail0 > 0) {
    launch_line_tail(tail, sc, s);
  } else {
    V c = view(L - 1);
    launch_coarse_solve_t(c, h->Ainv, h->cmap, h->ncoarse, sc, s);
  }
  for (int l = lk - 1; l >= 0; --l) {
    launch_prolong_lt(tview(l), view(l + 1), om, sc, s);
    const int npost = steps(l, true);
    for (int it = 0; it < npost; ++it)
      step(l, true, false, it == 0, do_rz && l == 0 && it == npost - 1);
  }
  if (do_rz && !rz_done) {
    const V f = view(0);
    launch_dot_rz_t<T, T>(f.nx, f.ny, f.pitch, f.b, f.x, flexible, sc, h->part, s);
  }
}

// V-cycle of the handle's precision on level 0: b = r (or its FP32 copy), x = z
void enqueue_vcycle(scf_proj* h, Scalars* sc, bool do_rz, cudaStream_t s) {
  if (!h->mixed) {
    auto view = [h](int l) { return view64(h, l); };
    auto buf = [h](int l, int i) { return buf64(h, l, i); };
    if (h->line) {
      auto tview = [h](int l) { return h->t64[l]; };
      enqueue_vcycle_line_t<double, double>(h, view, tview, h->ltail64, sc, do_rz, 0, s);
    } else {
      enqueue_vcycle_t(h, view, buf, h->tail64, sc, do_rz, 0, s);
    }
  } else {
    auto view = [h](int l) {
      MgF v = h->mix[l];
      if (l == 0) v.b = h->r32;
      return v;
    };
    auto buf = [h](int l, int i) { return buf32(h, l, i); };
    if (h->line) {
      auto tview = [h](int l) { return h->t32[l]; };
      enqueue_vcycle_line_t<float, bf16>(h, view, tview, h->ltail32, sc, do_rz, 1, s);
    } else {
      enqueue_vcycle_t(h, view, buf, h->tail32, sc, do_rz, 1, s);
    }
  }
}

// transposed operator of every level for the line smoother
template <class T, class CT>
void enqueue_line_setup_t(const std::vector<MgView<T, CT, T>>& nat,
                          const std::vector<MgView<T, CT, T>>& tr, cudaStream_t s) {
  for (size_t l = 0; l < nat.size(); ++l) {
    const MgView<T, CT, T>& f = nat[l];
    const MgView<T, CT, T>& t = tr[l];
    launch_transpose<CT>(f.cN, f.nx, f.ny, f.pitch, const_cast<CT*>(t.cE), t.pitch, nullptr, s);
    launch_transpose<CT>(f.cE, f.nx, f.ny, f.pitch, const_cast<CT*>(t.cN), t.pitch, nullptr, s);
    launch_transpose<T>(f.dg, f.nx, f.ny, f.pitch, const_cast<T*>(t.dg), t.pitch, nullptr, s);
    launch_transpose<T>(f.di, f.nx, f.ny, f.pitch, const_cast<T*>(t.di), t.pitch, nullptr, s);
  }
}

// assembly of the fine operator and setup of the whole hierarchy
// fork: mixed levels are converted on `aux` (one projection on the GPU); a
// batch branch keeps everything on `s`, since its branches already overlap.
void enqueue_setup(scf_proj* h, Scalars* sc, cudaStream_t s, bool fork = true) {
  const size_t nl = h->lev.size();
  // mixed: level l's largest coupling and FP32/BF16 copy on `aux` once level
  // l is built (an event per level), joined before the line setup
  cudaStream_t cs = fork ? h->aux : s;
  auto convert = [&](size_t l) {
    if (fork) {
      cudaEventRecord(h->lev_ev[l], s);
      cudaStreamWaitEvent(h->aux, h->lev_ev[l], 0);
    }
    launch_max_coupling(h->lev[l], h->maxbits + l, cs);
    launch_to_mixed(h->lev[l], h->mix[l], h->maxbits + l, h->cscale + l, cs);
  };
  launch_assemble(h->fin, h->lev[0], sc, s);
  // FP64 inverse diagonals serve the FP64 smoothers only; the mixed setup's
  // largest couplings restart from zero
  launch_excess(h->lev[0], h->mixed ? nullptr : h->di64[0], h->mixed ? h->maxbits : nullptr,
                (int)nl, sc, s);
  if (h->mixed && fork) convert(0);
  for (size_t l = 1; l < nl; ++l) {
    launch_coarsen(h->lev[l - 1], h->lev[l], h->mixed ? nullptr : h->di64[l], s);
    if (h->mixed && fork) convert(l);
  }
  launch_coarse_setup(h->lev.back(), h->Ainv, h->cmap, h->ncoarse, s);
  if (h->mixed && !fork)
    for (size_t l = 0; l < nl; ++l) convert(l);
  if (h->mixed && fork) {
    cudaEventRecord(h->aux_done, h->aux);
    cudaStreamWaitEvent(s, h->aux_done, 0);
  }
  if (h->line) {
    if (h->mixed) {
      enqueue_line_setup_t(h->mix, h->t32, s);
    } else {
      std::vector<MgD> nat;
      for (size_t l = 0; l < h->lev.size(); ++l) nat.push_back(view64(h, l));
      enqueue_line_setup_t(nat, h->t64, s);
      for (size_t l = 0; l < h->lf64n.size(); ++l) {
        launch_line_factor<double, double>(nat[l], h->lf64n[l], s);
        launch_line_factor<double, double>(h->t64[l], h->lf64t[l], s);
      }
    }
  }
}

// ---- the FP64 multigrid as a preconditioner of another 5-point operator ----
// Fine level from an external operator: the symmetric part of its couplings
// (clamped at zero, so every level stays an M-matrix) and its diagonal.
__global__ void k_mgpre_level0(LevelView L, const double* __restrict__ P,
                               const double* __restrict__ W, const double* __restrict__ E,
                               const double* __restrict__ S, const double* __restrict__ N) {
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= L.nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < L.ny; iy += gridDim.y * 8) {
    const size_t g = (size_t)iy * L.pitch + ix;
    const double d = P[g];
    L.dg[g] = d > 0.0 ? d : -1.0;
    L.cE[g] = ix + 1 < L.nx ? fmax(0.0, -0.5 * (E[g] + W[g + 1])) : 0.0;
    L.cN[g] = iy + 1 < L.ny ? fmax(0.0, -0.5 * (N[g] + S[g + L.pitch])) : 0.0;
  }
}

// the hierarchy below the fine level (enqueue_setup without the assembly)
void enqueue_setup_levels(scf_proj* h, Scalars* sc, cudaStream_t s) {
  const size_t nl = h->lev.size();
  launch_excess(h->lev[0], h->di64[0], nullptr, (int)nl, sc, s);
  for (size_t l = 1; l < nl; ++l) launch_coarsen(h->lev[l - 1], h->lev[l], h->di64[l], s);
  launch_coarse_setup(h->lev.back(), h->Ainv, h->cmap, h->ncoarse, s);
}

// transposed levels of the line smoother (allocated once, on first use)
int alloc_line(scf_proj* h) {
  if (h->line_alloc) return SCF_OK;
  int rc;
  for (size_t l = 0; l < h->lev.size(); ++l) {
    const int nx = h->lev[l].nx, ny = h->lev[l].ny;
    const int pt = (ny + 2 + 31) / 32 * 32;  // transposed: ny columns, nx rows
    if (!h->mixed) {
      MgD v{};
      v.nx = ny; v.ny = nx; v.pitch = pt;
      double *ce, *cn, *dg, *di, *x, *b;
      if ((rc = level_array(h, nx, pt, &ce)) || (rc = level_array(h, nx, pt, &cn)) ||
          (rc = level_array(h, nx, pt, &dg)) || (rc = level_array(h, nx, pt, &di)) ||
          (rc = level_array(h, nx, pt, &x)) || (rc = level_array(h, nx, pt, &b)))
        return rc;
      v.cE = ce; v.cN = cn; v.dg = dg; v.di = di; v.x = x; v.b = b;
      v.xin = nullptr; v.csp = nullptr;
      h->t64.push_back(v);
      // factors of the levels relaxed by kernels (the tail solves its own lines)
      const int lk = h->ltail0 > 0 ? h->ltail0 : (int)h->lev.size() - 1;
      if ((int)l < lk) {
        auto factors = [&](int rows, int len, int pitch, LineFactors<double>* F) {
          F->nth = line_threads(len, nullptr);
          double** arr[5] = {&F->inv, &F->ga, &F->cp, &F->S, &F->tr};
          for (auto a : arr)
            if (int e = level_array(h, rows, pitch, a)) return e;
          return dev_alloc(h, (void**)&F->thr,
                           sizeof(double) * (size_t)rows * F->nth * kLineThreadSlots);
        };
        LineFactors<double> fn{}, ft{};
        if ((rc = factors(ny, nx, h->lev[l].pitch, &fn)) || (rc = factors(nx, ny, pt, &ft)))
          return rc;
        h->lf64n.push_back(fn);
        h->lf64t.push_back(ft);
      }
    } else {
      MgF v{};
      v.nx = ny; v.ny = nx; v.pitch = pt;
      bf16 *ce, *cn;
      float *dg, *di, *x, *b;
      if ((rc = level_array(h, nx, pt, &ce)) || (rc = level_array(h, nx, pt, &cn)) ||
          (rc = level_array(h, nx, pt, &dg)) || (rc = level_array(h, nx, pt, &di)) ||
          (rc = level_array(h, nx, pt, &x)) || (rc = level_array(h, nx, pt, &b)))
        return rc;
      v.cE = ce; v.cN = cn; v.dg = dg; v.di = di; v.x = x; v.b = b;
      v.xin = nullptr; v.csp = h->mix[l].csp;
      h->t32.push_back(v);
    }
  }
  h->line_alloc = true;
  return SCF_OK;
}

// one PCG iteration: z = M r, beta, p = z + beta p_old, q = A p, alpha,
// x += alpha p, r -= alpha q (and the flexible cross term), convergence test
void enqueue_iteration(scf_proj* h, const double* pold, double* pnew, unsigned long long cond,
                       cudaStream_t s) {
  LevelView L0 = h->lev[0];
  const int zf = final_buf(h, 0);
  enqueue_vcycle(h, h->sc, true, s);
  if (!h->mixed) {
    launch_pupdate_spmv_t<double>(L0, buf64(h, 0, zf), pold, pnew, h->q, h->sc, h->part, s);
    launch_update_xr(L0, h->xsol, pnew, L0.b, nullptr, nullptr, h->q, h->sc, h->part, cond, s);
  } else {
    // the FP32 preconditioner's search direction is FP32 (in the same buffers)
    const float* z = buf32(h, 0, zf);
    const float* po = reinterpret_cast<const float*>(pold);
    float* pn = reinterpret_cast<float*>(pnew);
    launch_pupdate_spmv_t<float>(L0, z, po, pn, h->q, h->sc, h->part, s);
    launch_update_xr(L0, h->xsol, (const float*)pn, L0.b, h->r32, z, h->q, h->sc, h->part, cond, s);
  }
}

void enqueue_body(scf_proj* h, unsigned long long cond, cudaStream_t s) {
  enqueue_iteration(h, h->pA, h->pB, cond, s);
  enqueue_iteration(h, h->pB, h->pA, cond, s);
}

int build_graph(scf_proj* h) {
  destroy_graph(h);
  if (h->opts.flags & SCF_FLAG_NO_GRAPH) return SCF_OK;
  cudaStream_t cs = nullptr;
  CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  bool ok = false;
  do {  // preferred: conditional while node
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) break;
    cudaGraphConditionalHandle handle;
    if (cudaGraphConditionalHandleCreate(&handle, g, 1, cudaGraphCondAssignDefault) !=
        cudaSuccess) {
      cudaGraphDestroy(g);
      break;
    }
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = handle;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) != cudaSuccess) {
      cudaGraphDestroy(g);
      break;
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    if (cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      cudaGraphDestroy(g);
      break;
    }
    const long long l0 = g_launches;
    enqueue_body(h, (unsigned long long)handle, cs);
    h->body_launches = g_launches - l0;
    cudaGraph_t captured = nullptr;
    if (cudaStreamEndCapture(cs, &captured) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphDestroy(g);
      break;
    }
    cudaGraphExec_t ge = nullptr;
    if (cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphDestroy(g);
      break;
    }
    h->graph = g;
    h->gexec = ge;
    h->graph_cond = true;
    ok = true;
  } while (0);
  if (!ok) {  // fallback: graph of the loop body, relaunched and polled from the host
    cudaGetLastError();
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
    const long long l0 = g_launches;
    enqueue_body(h, 0ull, cs);
    h->body_launches = g_launches - l0;
    CK(cudaStreamEndCapture(cs, &h->body_graph));
    CK(cudaGraphInstantiate(&h->body_exec, h->body_graph, 0));
    h->graph_cond = false;
  }
  cudaStreamDestroy(cs);
  return SCF_OK;
}

// Add one instance's whole projection to the batch graph g as an independent
// branch: scalars reset, operator setup, right-hand side, the PCG loop as a
// conditional WHILE node (body: two iterations, as in build_graph), the
// correction and the copy of the scalars to pinned host memory.
struct BatchIO {
  const double *ustar = nullptr, *vstar = nullptr;
  double vb = 0.0;
  double *Pp = nullptr, *p = nullptr, *u = nullptr, *v = nullptr, *mres = nullptr;
  bool set = false;
};

int add_batch_branch(scf_proj* h, const BatchIO& io, cudaGraph_t g, cudaStream_t cs,
                     cudaStream_t cs2, long long* once, long long* body_launches) {
  if (cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) !=
      cudaSuccess)
    return SCF_ERR_CUDA;
  int rc = SCF_OK;
  const long long l0 = g_launches;
  long long lb = 0;
  do {
    cudaMemsetAsync(h->sc, 0, sizeof(Scalars), cs);
    enqueue_setup(h, h->sc, cs, false);
    LevelView L0 = h->lev[0];
    launch_rhs(h->fin, io.ustar, io.vstar, io.vb, L0, h->bvec, L0.b, h->r32, h->xsol, h->sc,
               h->part, h->opts.rtol, h->opts.maxit, cs);
    // the conditional node, added by hand at the capture's current position
    cudaStreamCaptureStatus cst;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaGraph_t cg = nullptr;
    if (cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &ndeps) != cudaSuccess ||
        cst != cudaStreamCaptureStatusActive) {
      rc = SCF_ERR_CUDA;
      break;
    }
    cudaGraphConditionalHandle handle;
    if (cudaGraphConditionalHandleCreate(&handle, cg, 1, cudaGraphCondAssignDefault) !=
        cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = handle;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &np) != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    if (cudaStreamBeginCaptureToGraph(cs2, body, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    const long long b0 = g_launches;
    enqueue_body(h, (unsigned long long)handle, cs2);
    lb = g_launches - b0;
    cudaGraph_t captured = nullptr;
    if (cudaStreamEndCapture(cs2, &captured) != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if (cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1,
                                            cudaStreamSetCaptureDependencies) !=
        cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    launch_final_solution(h->fin, L0, h->xsol, h->bvec, io.ustar, io.vstar, io.Pp, io.p, io.u,
                          io.v, 1, h->sc, h->part, cs);
    launch_final_mres(h->fin, io.vb, io.u, io.v, io.mres, h->sc, h->part, cs);
    launch_final_zero(h->fin, io.p, io.u, io.v, cs);
    cudaMemcpyAsync(h->sc_host, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, cs);
  } while (0);
  *body_launches = lb;
  *once = g_launches - l0 - lb;
  cudaGraph_t out = nullptr;
  const cudaError_t e = cudaStreamEndCapture(cs, &out);
  if (rc == SCF_OK && e != cudaSuccess) rc = SCF_ERR_CUDA;
  if (rc != SCF_OK) cudaGetLastError();
  return rc;
}

int read_scalars(scf_proj* h) {
  CK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return SCF_OK;
}

// run the PCG loop (right-hand side already in place)
int run_pcg(scf_proj* h) {
  if (h->graph_cond && h->gexec) {
    CK(cudaGraphLaunch(h->gexec, h->stream));
    return SCF_OK;
  }
  const int maxit = h->opts.maxit;
  int launched = 0;
  while (launched < maxit) {
    const int chunk = 4;  // body launches (2 iterations each) between polls
    for (int c = 0; c < chunk && launched < maxit; ++c) {
      if (h->body_exec) {
        CK(cudaGraphLaunch(h->body_exec, h->stream));
        ++h->body_runs;
      } else {
        enqueue_body(h, 0ull, h->stream);
        CK(cudaGetLastError());
      }
      launched += 2;
    }
    int rc = read_scalars(h);
    if (rc) return rc;
    if (h->sc_host->done) break;
  }
  return SCF_OK;
}

// Flexible PCG with the learned preconditioner (mixed handles): z = sigma *
// U-Net(r) while each iteration reduces ||r|| by at least kLearnedRatio,
// then the mixed V-cycle for the rest of the solve.  Host-polled (one
// scalar read per iteration decides the preconditioner of the next).
constexpr double kLearnedRatio = 0.6;

int run_learned(scf_proj* h, int* nn_iters, int* fell_back) {
  cudaStream_t s = h->stream;
  LevelView L0 = h->lev[0];
  const int zf = final_buf(h, 0);
  float* z = buf32(h, 0, zf);
  int rc = read_scalars(h);
  if (rc) return rc;
  double rr_prev = h->sc_host->rr;
  bool use_nn = true;
  *nn_iters = 0;
  *fell_back = 0;
  double* pold = h->pA;
  double* pnew = h->pB;
  for (int it = 0; it < h->opts.maxit && !h->sc_host->done; ++it) {
    if (use_nn) {
      h->net->features(0, L0.nx, L0.ny, L0.pitch, L0.b, L0.cE, L0.cN, L0.dg, h->net_sigma, s);
      h->net->forward(s);
      h->net->correction(L0.nx, L0.ny, L0.pitch, L0.dg, h->net_sigma, z, s);
      launch_dot_rz_t<float, float>(L0.nx, L0.ny, L0.pitch, h->r32, z, 1, h->sc, h->part, s);
    } else {
      enqueue_vcycle(h, h->sc, true, s);
    }
    float* pn = reinterpret_cast<float*>(pnew);
    launch_pupdate_spmv_t<float>(L0, z, reinterpret_cast<const float*>(pold), pn, h->q, h->sc,
                                 h->part, s);
    launch_update_xr(L0, h->xsol, (const float*)pn, L0.b, h->r32, z, h->q, h->sc, h->part, 0ull, s);
    CK(cudaGetLastError());
    std::swap(pold, pnew);
    if ((rc = read_scalars(h))) return rc;
    const double rr = h->sc_host->rr;
    if (use_nn) {
      ++*nn_iters;
      if (!(rr <= kLearnedRatio * kLearnedRatio * rr_prev)) {
        use_nn = false;
        *fell_back = 1;
      }
    }
    rr_prev = rr;
  }
  return SCF_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) return 0.f;
  return ms;
}

template <class T>
int put(scf_proj* h, T** dst, const T* src, size_t n) {
  if (!src) return SCF_ERR_ARG;
  if (h->devptrs) {
    *dst = const_cast<T*>(src);
    return SCF_OK;
  }
  CK(cudaMemcpyAsync(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice, h->stream));
  return SCF_OK;
}

bool learned(const scf_proj* h) { return h->opts.precond == SCF_PRECOND_LEARNED; }

int solve_common(scf_proj* h, const double* ustar, const double* vstar, double vb, double* Pp,
                 double* p, double* u, double* v, double* mres, scf_stats* st, bool correct) {
  if (!h) return SCF_ERR_ARG;
  if (!h->assembled) return SCF_ERR_STATE;
  if (learned(h) && !h->net) return SCF_ERR_STATE;
  if (!ustar || !vstar) return SCF_ERR_ARG;
  if (correct && (!p || !u || !v || !mres)) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  const int nx = h->nx, ny = h->ny;
  const size_t n0 = (size_t)(nx + 2) * (ny + 2), n1 = (size_t)nx * ny;
  cudaStream_t s = h->stream;
  const long long l0 = g_launches;
  h->body_runs = 0;
  // host mode: the input copies go on the copy stream, so they overlap the
  // operator setup that assemble left running on the solver stream (the
  // staging buffers are idle: every solve ends with a synchronisation)
  cudaStream_t cs = h->devptrs ? s : h->copy_stream;
  CK(cudaEventRecord(h->ev[0], cs));
  const double *dus = ustar, *dvs = vstar;
  double *dPp = Pp, *dp = p, *du = u, *dv = v, *dm = mres;
  bool late = false;  // copies that only the correction waits for
  if (!h->devptrs) {
    CK(cudaMemcpyAsync(h->st_us, ustar, n0 * 8, cudaMemcpyHostToDevice, cs));
    CK(cudaMemcpyAsync(h->st_vs, vstar, n0 * 8, cudaMemcpyHostToDevice, cs));
    dus = h->st_us; dvs = h->st_vs;
    dPp = Pp ? h->st_Pp : nullptr;
    CK(cudaEventRecord(h->copy_done, cs));
    CK(cudaStreamWaitEvent(s, h->copy_done, 0));
    // the rest is read by the correction only: these copies run during the solve
    if (correct) {
      CK(cudaMemcpyAsync(h->st_p, p, n0 * 8, cudaMemcpyHostToDevice, cs));
      CK(cudaMemcpyAsync(h->st_u, u, n0 * 8, cudaMemcpyHostToDevice, cs));
      CK(cudaMemcpyAsync(h->st_v, v, n0 * 8, cudaMemcpyHostToDevice, cs));
      dp = h->st_p; du = h->st_u; dv = h->st_v; dm = h->st_mres;
      late = true;
    }
    if (h->late_pending) {
      for (const auto& e : h->late)
        CK(cudaMemcpyAsync(e.dst, e.src, e.bytes, cudaMemcpyHostToDevice, cs));
      h->late_pending = false;
      late = true;
    }
    if (late) CK(cudaEventRecord(h->late_done, cs));
  }
  CK(cudaEventRecord(h->ev[1], cs));
  LevelView L0 = h->lev[0];
  // the NaN flag of a previous solve must not leak into this one
  CK(cudaMemsetAsync(&h->sc->nan, 0, sizeof(int), s));
  launch_rhs(h->fin, dus, dvs, vb, L0, h->bvec, L0.b, h->r32, h->xsol, h->sc, h->part,
             h->opts.rtol, h->opts.maxit, s);
  CK(cudaGetLastError());
  int nn_iters = 0, fell_back = 0;
  int rc = learned(h) ? run_learned(h, &nn_iters, &fell_back) : run_pcg(h);
  if (rc) return rc;
  CK(cudaEventRecord(h->ev[2], s));
  if (late) CK(cudaStreamWaitEvent(s, h->late_done, 0));
  launch_final_solution(h->fin, L0, h->xsol, h->bvec, dus, dvs, dPp, dp, du, dv, correct ? 1 : 0,
                        h->sc, h->part, s);
  if (correct) {
    launch_final_mres(h->fin, vb, du, dv, dm, h->sc, h->part, s);
    launch_final_zero(h->fin, dp, du, dv, s);
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->ev[3], s));
  if (!h->devptrs) {
    if (Pp) CK(cudaMemcpyAsync(Pp, h->st_Pp, n0 * 8, cudaMemcpyDeviceToHost, s));
    if (correct) {
      CK(cudaMemcpyAsync(p, h->st_p, n0 * 8, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(u, h->st_u, n0 * 8, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(v, h->st_v, n0 * 8, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(mres, h->st_mres, n1 * 8, cudaMemcpyDeviceToHost, s));
    }
  }
  CK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(h->ev[4], s));
  CK(cudaStreamSynchronize(s));
  const Scalars& S = *h->sc_host;
  int status = S.status;
  if (S.nan || S.anan) status = SCF_ERR_NAN;
  if (st) {
    st->iters = S.iter;
    st->status = status;
    st->levels = (int)h->lev.size();
    st->fallbacks = fell_back;
    st->learned_iters = nn_iters;
    st->smoother = h->line ? SCF_SMOOTH_LINE : SCF_SMOOTH_POINT;
    st->bnorm = sqrt(S.bnorm2);
    st->relres = S.bnorm2 > 0 ? sqrt(S.rr / S.bnorm2) : 0.0;
    st->relres_true = S.bnorm2 > 0 ? sqrt(S.res_true2 / S.bnorm2) : 0.0;
    st->mres_max = correct ? S.mres_max : 0.0;
    st->ms_h2d = elapsed(h->ev[0], h->ev[1]);
    st->ms_solve = elapsed(h->ev[1], h->ev[2]);
    st->ms_correct = elapsed(h->ev[2], h->ev[3]);
    st->ms_d2h = elapsed(h->ev[3], h->ev[4]);
    st->ms_total = elapsed(h->ev[0], h->ev[4]);
    st->ms_assemble = 0.0;
    // direct launches, plus the kernel nodes of every executed loop body
    // (k_update_xr counts two per body execution in the loop guard)
    long long n = h->pending_launches + (g_launches - l0);
    if (h->graph_cond && h->gexec && !learned(h)) n += (long long)(S.pad[0] / 2) * h->body_launches;
    n += h->body_runs * h->body_launches;
    st->launches = (int)n;
    st->asym_faces = S.asym_faces;
  }
  h->pending_launches = 0;
  return status == kOk ? SCF_OK : status;
}

}  // namespace

extern "C" {

void scf_opts_default(scf_opts* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->precision = SCF_PREC_FP64;
  o->flags = 0;
  o->device = 0;
  o->maxit = 200;
  o->rtol = 1.0e-8;
  o->npre = 2;
  o->npost = 2;
  o->omega = 1.9;
  o->coarse_max = 64;
  o->smoother = SCF_SMOOTH_AUTO;
}

int scf_diag_divide(const double* a, const double* b, double* q, int64_t n, int device) {
  if (n < 0 || (n > 0 && (!a || !b || !q))) return SCF_ERR_ARG;
  if (n == 0) return SCF_OK;
  CK(cudaSetDevice(device));
  double* d = nullptr;
  const size_t bytes = (size_t)n * 8;
  CK(cudaMalloc(&d, 3 * bytes));
  int rc = SCF_OK;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(d);
    return SCF_ERR_CUDA;
  }
  if (cudaMemcpyAsync(d, a, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(d + n, b, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = SCF_ERR_CUDA;
  if (rc == SCF_OK) {
    launch_divide(d, d + n, d + 2 * n, (long long)n, s);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(q, d + 2 * n, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = SCF_ERR_CUDA;
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  cudaFree(d);
  return rc;
}

int scf_diag_sqrt(const double* a, double* q, int64_t n, int device) {
  if (n < 0 || (n > 0 && (!a || !q))) return SCF_ERR_ARG;
  if (n == 0) return SCF_OK;
  CK(cudaSetDevice(device));
  double* d = nullptr;
  const size_t bytes = (size_t)n * 8;
  CK(cudaMalloc(&d, 2 * bytes));
  int rc = SCF_OK;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(d);
    return SCF_ERR_CUDA;
  }
  if (cudaMemcpyAsync(d, a, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = SCF_ERR_CUDA;
  if (rc == SCF_OK) {
    launch_sqrt(d, d + n, (long long)n, s);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(q, d + n, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = SCF_ERR_CUDA;
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  cudaFree(d);
  return rc;
}

const char* scf_strerror(int code) {
  switch (code) {
    case SCF_OK: return "ok";
    case SCF_ERR_ARG: return "invalid argument";
    case SCF_ERR_CUDA: return "CUDA error";
    case SCF_ERR_NAN: return "NaN or Inf in operator, right-hand side or iterate";
    case SCF_ERR_NOT_CONVERGED: return "maximum iterations reached before tolerance";
    case SCF_ERR_STALL: return "residual stalled";
    case SCF_ERR_TIMEOUT: return "bounded device wait ran out";
    case SCF_ERR_STATE: return "call order (grid, geometry and assemble must come first)";
    case SCF_ERR_NOMEM: return "device memory allocation failed";
    case SCF_ERR_IO: return "file could not be opened or written";
    default: return "unknown status";
  }
}

int scf_proj_create(scf_proj** out, int nx, int ny, const scf_opts* opts) {
  if (!out) return SCF_ERR_ARG;
  *out = nullptr;
  if (nx < 2 || ny < 2 || nx > (1 << 16) || ny > (1 << 16)) return SCF_ERR_ARG;
  scf_opts o;
  if (opts) o = *opts; else scf_opts_default(&o);
  if (o.precision != SCF_PREC_FP64 && o.precision != SCF_PREC_MIXED) return SCF_ERR_ARG;
  if (o.maxit < 1 || o.npre < 1 || o.npost < 1 || o.npre > 8 || o.npost > 8 || !(o.rtol >= 0.0))
    return SCF_ERR_ARG;
  if (o.coarse_max < 1 || o.coarse_max > kMaxCoarse) return SCF_ERR_ARG;
  if (o.coarse_sweeps < 0 || o.coarse_sweeps > 8 || o.coarse_from < 0 || o.coarse_from > 64)
    return SCF_ERR_ARG;
  if (!(o.omega > 0.0 && o.omega < 2.0)) return SCF_ERR_ARG;
  if (o.smoother != SCF_SMOOTH_AUTO && o.smoother != SCF_SMOOTH_POINT &&
      o.smoother != SCF_SMOOTH_LINE)
    return SCF_ERR_ARG;
  if (o.smoother == SCF_SMOOTH_LINE && (nx > kLineMaxLen || ny > kLineMaxLen)) return SCF_ERR_ARG;
  if (o.precond != SCF_PRECOND_MG && o.precond != SCF_PRECOND_LEARNED) return SCF_ERR_ARG;
  if (o.precond == SCF_PRECOND_LEARNED && o.precision != SCF_PREC_MIXED) return SCF_ERR_ARG;
  scf_proj* h = new (std::nothrow) scf_proj();
  if (!h) return SCF_ERR_NOMEM;
  h->nx = nx; h->ny = ny; h->opts = o;
  h->device = o.device;
  h->devptrs = (o.flags & SCF_FLAG_DEVICE_PTRS) != 0;
  h->mixed = o.precision == SCF_PREC_MIXED;
  int rc = SCF_OK;
  auto fail = [&](int code) { scf_proj_destroy(h); return code; };
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(SCF_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(SCF_ERR_CUDA);
  h->own_stream = true;
  if (cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->copy_done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->late_done, cudaEventDisableTiming) != cudaSuccess)
    return fail(SCF_ERR_CUDA);
  if (h->mixed) {
    if (cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->aux_done, cudaEventDisableTiming) != cudaSuccess)
      return fail(SCF_ERR_CUDA);
    for (auto& e : h->lev_ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
        return fail(SCF_ERR_CUDA);
  }
  for (auto& e : h->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(SCF_ERR_CUDA);
  // FP64 multigrid levels
  int lx = nx, ly = ny;
  while (true) {
    LevelView L{};
    L.nx = lx; L.ny = ly; L.pitch = round_up(lx + 2, 32);
    double** arrs[6] = {&L.cE, &L.cN, &L.dg, &L.ex, &L.x, &L.b};
    for (auto a : arrs)
      if ((rc = level_array(h, ly, L.pitch, a))) return fail(rc);
    double* di = nullptr;
    if ((rc = level_array(h, ly, L.pitch, &di))) return fail(rc);
    double* x2 = nullptr;
    if ((rc = level_array(h, ly, L.pitch, &x2))) return fail(rc);
    if (h->lev.empty()) {  // the fine level: the rows' own west / south entries
      if ((rc = level_array(h, ly, L.pitch, &L.wW)) || (rc = level_array(h, ly, L.pitch, &L.wS)) ||
          (rc = dev_alloc(h, (void**)&L.arow, sizeof(int) * (size_t)ly)))
        return fail(rc);
      // mixed: the float pairs of the operator for the FP32-direction SpMV
      if (h->mixed &&
          ((rc = level_array(h, ly, L.pitch, &L.fE)) || (rc = level_array(h, ly, L.pitch, &L.fN)) ||
           (rc = level_array(h, ly, L.pitch, &L.fD))))
        return fail(rc);
    }
    h->lev.push_back(L);
    h->di64.push_back(di);
    h->x2_64.push_back(x2);
    if ((long)lx * ly <= o.coarse_max || (lx == 1 && ly == 1) || h->lev.size() >= 30) break;
    lx = (lx + 1) / 2; ly = (ly + 1) / 2;
  }
  const int nlev = (int)h->lev.size();
  if ((rc = dev_alloc(h, (void**)&h->cscale, sizeof(float) * nlev))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->maxbits, sizeof(unsigned) * nlev))) return fail(rc);
  if (h->mixed) {
    for (int l = 0; l < nlev; ++l) {
      const LevelView& F = h->lev[l];
      bf16 *ce = nullptr, *cn = nullptr;
      float *dg = nullptr, *di = nullptr, *x = nullptr, *x2 = nullptr, *b = nullptr;
      if ((rc = level_array(h, F.ny, F.pitch, &ce)) || (rc = level_array(h, F.ny, F.pitch, &cn)) ||
          (rc = level_array(h, F.ny, F.pitch, &dg)) || (rc = level_array(h, F.ny, F.pitch, &di)) ||
          (rc = level_array(h, F.ny, F.pitch, &x)) || (rc = level_array(h, F.ny, F.pitch, &x2)) ||
          (rc = level_array(h, F.ny, F.pitch, &b)))
        return fail(rc);
      MgF v{};
      v.nx = F.nx; v.ny = F.ny; v.pitch = F.pitch;
      v.cE = ce; v.cN = cn; v.dg = dg; v.di = di;
      v.x = x; v.b = b; v.xin = nullptr; v.csp = h->cscale + l;
      h->mix.push_back(v);
      h->x2_32.push_back(x2);
    }
    if ((rc = level_array(h, ny, h->lev[0].pitch, &h->r32))) return fail(rc);
    // tensor maps of the TMA-staged sweep (levels of at least 128 x 64 cells),
    // encoded on the host, kept in device memory
    h->dmaps.assign(nlev, nullptr);
    h->tma.assign(nlev, 0);
    for (int l = 0; l < nlev; ++l) {
      const MgF& M = h->mix[l];
      if (M.nx < 128 || M.ny < 64) continue;
      alignas(64) CUtensorMap hm[kSweepMaps];
      float* const xb[2] = {buf32(h, l, 0), buf32(h, l, 1)};
      if (!make_sweep_maps(M, xb, l == 0 ? h->r32 : M.b, hm)) continue;
      if ((rc = dev_alloc(h, (void**)&h->dmaps[l], sizeof(hm)))) return fail(rc);
      if (cudaMemcpyAsync(h->dmaps[l], hm, sizeof(hm), cudaMemcpyHostToDevice, h->stream) !=
              cudaSuccess ||
          cudaStreamSynchronize(h->stream) != cudaSuccess)
        return fail(SCF_ERR_CUDA);
      h->tma[l] = 1;
    }
  }
  const int P0 = h->lev[0].pitch;
  double** pv[5] = {&h->xsol, &h->pA, &h->pB, &h->q, &h->bvec};
  for (auto a : pv)
    if ((rc = level_array(h, ny, P0, a))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->Ainv, sizeof(double) * kMaxCoarse * kMaxCoarse))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->cmap, sizeof(int) * kMaxCoarse))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->ncoarse, sizeof(int)))) return fail(rc);
  // the single-CTA tail: the first level >= 1 with at most tail_cells() cells
  // whose levels fit one CTA's shared memory (ragged grids may need a later one)
  // (a 64 x 64 level in the FP32 tail measured no faster than its own
  // launches: the tail's phases are latency-bound)
  if (!getenv("SCF_NO_TAIL")) {
    for (int l = 1; l < nlev; ++l) {
      if ((long)h->lev[l].nx * h->lev[l].ny > tail_cells() || nlev - l > kTailMaxLevels) continue;
      auto fill = [&](auto& d, auto view) {
        d.n = nlev - l;
        for (int k = 0; k < d.n; ++k) d.lv[k] = view(l + k);
        d.npre = o.npre; d.npost = o.npost;
        set_tail_coarse(d, o, l);
        d.omega = (decltype(d.omega))o.omega;
        d.Ainv = h->Ainv; d.cmap = h->cmap; d.nc = h->ncoarse;
        return tail_prepare(d);
      };
      const int bad = h->mixed ? fill(h->tail32, [h](int k) { return h->mix[k]; })
                               : fill(h->tail64, [h](int k) { return view64(h, k); });
      if (!bad) { h->tail0 = l; break; }
    }
  }
  // the single-CTA tail of the line smoother, chosen the same way; its FP32
  // lines are solved by a warp each (up to 64 cells), so FP32 tails reach
  // 64 x 64 levels
  if (o.smoother != SCF_SMOOTH_POINT && !getenv("SCF_NO_TAIL")) {
    const long lcells = h->mixed && !getenv("SCF_TAIL_CELLS") ? kLineTailMaxCells32 : tail_cells();
    for (int l = 1; l < nlev; ++l) {
      if ((long)h->lev[l].nx * h->lev[l].ny > lcells || h->lev[l].nx > 64 || h->lev[l].ny > 64 ||
          nlev - l + 1 > kTailMaxLevels)
        continue;
      auto fill = [&](auto& d, auto view) {
        d.n = nlev - l;
        for (int k = 0; k < d.n; ++k) d.lv[k] = view(l + k);
        d.npre = o.npre; d.npost = o.npost;
        set_tail_coarse(d, o, l);
        d.omega = (decltype(d.omega))o.omega;
        d.Ainv = h->Ainv; d.cmap = h->cmap; d.nc = h->ncoarse;
        return line_tail_prepare(d);
      };
      int bad = h->mixed ? fill(h->ltail32, [h](int k) { return h->mix[k]; })
                         : fill(h->ltail64, [h](int k) { return view64(h, k); });
      if (!bad) { h->ltail0 = l; break; }
    }
  }
  if ((rc = dev_alloc(h, (void**)&h->aspect_bits, sizeof(unsigned)))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->sc, sizeof(Scalars)))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->sc_diag, sizeof(Scalars)))) return fail(rc);
  size_t nblk = 0;
  {
    dim3 g1 = grid_for(nx, ny, 1), g2 = grid_for(nx, ny, 2);
    nblk = (size_t)g1.x * g1.y;
    if ((size_t)g2.x * g2.y > nblk) nblk = (size_t)g2.x * g2.y;
    size_t tb = (size_t)((nx + 63) / 64) * ((ny + 31) / 32);
    if (tb > nblk) nblk = tb;
    // r.z reduction after a line-smoothed V-cycle: 32x8 blocks, at most 1024 rows of blocks
    const size_t gy = (size_t)(ny + 7) / 8;
    size_t rb = (size_t)((nx + 31) / 32) * (gy < 1024 ? gy : 1024);
    if (rb > nblk) nblk = rb;
    // direction update + SpMV
    int rows = 0;
    for (const dim3 g : {pupdate_grid(nx, ny, &rows), pupdate_ff_grid(nx, ny)})
      if ((size_t)g.x * g.y > nblk) nblk = (size_t)g.x * g.y;
    // r.z fused into the last line relaxation: one block per pair of rows
    const size_t lb = (size_t)(ny + 1) / 2;
    if (lb > nblk) nblk = lb;
  }
  if ((rc = dev_alloc(h, (void**)&h->part, sizeof(double) * (2 * nblk + 64)))) return fail(rc);
  if (cudaMallocHost((void**)&h->sc_host, sizeof(Scalars)) != cudaSuccess) return fail(SCF_ERR_NOMEM);
  memset(h->sc_host, 0, sizeof(Scalars));
  if (!h->devptrs) {  // Fortran-layout staging
    const size_t n0 = (size_t)(nx + 2) * (ny + 2), n1 = (size_t)nx * ny;
    struct { void** p; size_t b; } st[] = {
        {(void**)&h->st_dx, n1 * 8},  {(void**)&h->st_dy, n1 * 8},  {(void**)&h->st_dxU, n1 * 8},
        {(void**)&h->st_dyV, n1 * 8}, {(void**)&h->st_vof, n1 * 8}, {(void**)&h->st_phi, n1 * 8},
        {(void**)&h->st_vofS, n1 * 8}, {(void**)&h->st_nyS, n1 * 8}, {(void**)&h->st_WlLh, n1 * 8},
        {(void**)&h->st_aE, n0 * 8},  {(void**)&h->st_aW, n0 * 8},  {(void**)&h->st_aN, n0 * 8},
        {(void**)&h->st_aS, n0 * 8},  {(void**)&h->st_pp, n0 * 4},  {(void**)&h->st_pu, n0 * 4},
        {(void**)&h->st_pv, n0 * 4},  {(void**)&h->st_mu, n1 * 4},  {(void**)&h->st_mv, n1 * 4},
        {(void**)&h->st_vsu, n1 * 8}, {(void**)&h->st_vsv, n1 * 8}, {(void**)&h->st_DpU, n0 * 8},
        {(void**)&h->st_DpV, n0 * 8}, {(void**)&h->st_us, n0 * 8},  {(void**)&h->st_vs, n0 * 8},
        {(void**)&h->st_Pp, n0 * 8},  {(void**)&h->st_p, n0 * 8},   {(void**)&h->st_u, n0 * 8},
        {(void**)&h->st_v, n0 * 8},   {(void**)&h->st_mres, n1 * 8}};
    for (auto& e : st)
      if ((rc = dev_alloc(h, e.p, e.b))) return fail(rc);
  }
  h->fin.nx = nx; h->fin.ny = ny;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(SCF_ERR_CUDA);
  *out = h;
  return SCF_OK;
}

int scf_proj_destroy(scf_proj* h) {
  if (!h) return SCF_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  destroy_graph(h);
  delete h->net;
  for (void* p : h->allocs) cudaFree(p);
  if (h->sc_host) cudaFreeHost(h->sc_host);
  if (h->g_flag_host) cudaFreeHost(h->g_flag_host);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  if (h->copy_done) cudaEventDestroy(h->copy_done);
  if (h->late_done) cudaEventDestroy(h->late_done);
  if (h->aux) cudaStreamDestroy(h->aux);
  if (h->aux_done) cudaEventDestroy(h->aux_done);
  for (auto& e : h->lev_ev)
    if (e) cudaEventDestroy(e);
  delete h;
  return SCF_OK;
}

int scf_proj_set_stream(scf_proj* h, void* stream) {
  if (!h) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->stream = (cudaStream_t)stream;
  h->own_stream = false;
  return SCF_OK;
}

int scf_proj_set_grid(scf_proj* h, const double* dx, const double* dy, const double* dxU,
                      const double* dyV) {
  if (!h || !dx || !dy || !dxU || !dyV) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  const size_t n1 = (size_t)h->nx * h->ny;
  int rc;
  if ((rc = put(h, &h->st_dx, dx, n1)) || (rc = put(h, &h->st_dy, dy, n1)) ||
      (rc = put(h, &h->st_dxU, dxU, n1)) || (rc = put(h, &h->st_dyV, dyV, n1)))
    return rc;
  h->fin.dx = h->st_dx; h->fin.dy = h->st_dy; h->fin.dxU = h->st_dxU; h->fin.dyV = h->st_dyV;
  // smoother: lines when asked, or (auto) when some cell has an aspect ratio
  // above 2 (couplings 4x stronger along one axis), where red-black point
  // relaxation smooths poorly
  bool want = h->opts.smoother == SCF_SMOOTH_LINE;
  if (h->opts.smoother == SCF_SMOOTH_AUTO && h->nx <= kLineMaxLen && h->ny <= kLineMaxLen) {
    unsigned bits = 0;
    CK(cudaMemsetAsync(h->aspect_bits, 0, sizeof(unsigned), h->stream));
    launch_aspect(h->st_dx, h->st_dy, n1, h->aspect_bits, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&bits, h->aspect_bits, sizeof(unsigned), cudaMemcpyDeviceToHost,
                       h->stream));
    CK(cudaStreamSynchronize(h->stream));
    float aspect;
    memcpy(&aspect, &bits, sizeof(aspect));
    want = aspect > 2.0f;
  }
  if (want && (rc = alloc_line(h))) return rc;
  if (want != h->line) destroy_graph(h);
  h->line = want;
  CK(cudaStreamSynchronize(h->stream));
  h->have_grid = true;
  h->assembled = false;
  return SCF_OK;
}

int scf_proj_set_geometry(scf_proj* h, const double* vof, const double* phi, const double* vofS,
                          const double* nyS, const double* WlLh, const double* aE,
                          const double* aW, const double* aN, const double* aS,
                          const int32_t* posnu_p, const int32_t* posnu_u, const int32_t* moex_u,
                          const double* vofS_u, const int32_t* posnu_v, const int32_t* moex_v,
                          const double* vofS_v) {
  if (!h) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  const size_t n1 = (size_t)h->nx * h->ny, n0 = (size_t)(h->nx + 2) * (h->ny + 2);
  int rc;
  if ((rc = put(h, &h->st_vof, vof, n1)) || (rc = put(h, &h->st_phi, phi, n1)) ||
      (rc = put(h, &h->st_vofS, vofS, n1)) || (rc = put(h, &h->st_nyS, nyS, n1)) ||
      (rc = put(h, &h->st_WlLh, WlLh, n1)) || (rc = put(h, &h->st_aE, aE, n0)) ||
      (rc = put(h, &h->st_aW, aW, n0)) || (rc = put(h, &h->st_aN, aN, n0)) ||
      (rc = put(h, &h->st_aS, aS, n0)) || (rc = put(h, &h->st_pp, posnu_p, n0)))
    return rc;
  if (!posnu_u || !moex_u || !vofS_u || !posnu_v || !moex_v || !vofS_v) return SCF_ERR_ARG;
  if (h->devptrs) {
    h->st_pu = const_cast<int32_t*>(posnu_u); h->st_mu = const_cast<int32_t*>(moex_u);
    h->st_vsu = const_cast<double*>(vofS_u); h->st_pv = const_cast<int32_t*>(posnu_v);
    h->st_mv = const_cast<int32_t*>(moex_v); h->st_vsv = const_cast<double*>(vofS_v);
  } else {
    // read by the correction only: copied by the next solve, during its PCG
    h->late[0] = {h->st_pu, posnu_u, n0 * 4};
    h->late[1] = {h->st_mu, moex_u, n1 * 4};
    h->late[2] = {h->st_vsu, vofS_u, n1 * 8};
    h->late[3] = {h->st_pv, posnu_v, n0 * 4};
    h->late[4] = {h->st_mv, moex_v, n1 * 4};
    h->late[5] = {h->st_vsv, vofS_v, n1 * 8};
    h->late_pending = true;
  }
  FortranIn& f = h->fin;
  f.vof = h->st_vof; f.phi = h->st_phi; f.vofS = h->st_vofS; f.nyS = h->st_nyS;
  f.WlLh = h->st_WlLh; f.aE = h->st_aE; f.aW = h->st_aW; f.aN = h->st_aN; f.aS = h->st_aS;
  f.posnu_p = h->st_pp; f.posnu_u = h->st_pu; f.posnu_v = h->st_pv;
  f.moex_u = h->st_mu; f.moex_v = h->st_mv; f.vofS_u = h->st_vsu; f.vofS_v = h->st_vsv;
  CK(cudaStreamSynchronize(h->stream));
  h->have_geom = true;
  h->assembled = false;
  return SCF_OK;
}

int scf_proj_assemble(scf_proj* h, const double* DpU, const double* DpV, double betaP,
                      double betaM, int wb, int eb, int sb, int nb) {
  if (!h || !DpU || !DpV) return SCF_ERR_ARG;
  if (!h->have_grid || !h->have_geom) return SCF_ERR_STATE;
  if ((wb != 0 && wb != 1) || (eb != 0 && eb != 1) || (sb != 0 && sb != 1) || (nb != 0 && nb != 1))
    return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  const size_t n0 = (size_t)(h->nx + 2) * (h->ny + 2);
  int rc;
  if ((rc = put(h, &h->st_DpU, DpU, n0)) || (rc = put(h, &h->st_DpV, DpV, n0))) return rc;
  FortranIn& f = h->fin;
  f.DpU = h->st_DpU; f.DpV = h->st_DpV;
  f.betaP = betaP; f.betaM = betaM;
  f.wb = wb; f.eb = eb; f.sb = sb; f.nb = nb;
  cudaStream_t s = h->stream;
  // host mode: the caller may reuse DpU/DpV once their copies are done
  CK(cudaEventRecord(h->copy_done, s));
  CK(cudaMemsetAsync(h->sc, 0, sizeof(Scalars), s));
  const long long l0 = g_launches;
  enqueue_setup(h, h->sc, s);
  h->pending_launches += g_launches - l0;
  CK(cudaGetLastError());
  if (!h->gexec && !h->body_exec && !(h->opts.flags & SCF_FLAG_NO_GRAPH)) {
    if ((rc = build_graph(h))) return rc;
  }
  if (!h->devptrs) CK(cudaEventSynchronize(h->copy_done));
  h->assembled = true;
  return SCF_OK;
}

int scf_proj_poisson_solve(scf_proj* h, const double* ustar, const double* vstar, double vb,
                           double* Pp, scf_stats* st) {
  if (!Pp) return SCF_ERR_ARG;
  return solve_common(h, ustar, vstar, vb, Pp, nullptr, nullptr, nullptr, nullptr, st, false);
}

int scf_proj_update_puv(scf_proj* h, const double* ustar, const double* vstar, double vb,
                        double* Pp, double* p, double* u, double* v, double* mres,
                        scf_stats* st) {
  return solve_common(h, ustar, vstar, vb, Pp, p, u, v, mres, st, true);
}

int scf_proj_set_solid(scf_proj* h, const double* vof, const double* phi, const double* vofS,
                       const double* phiS, const double* nxS, const double* nyS,
                       const double* vofS_u, const double* vofS_v, int icorprob) {
  if (!h || !vof || !phi || !vofS || !phiS || !nxS || !nyS || !vofS_u || !vofS_v)
    return SCF_ERR_ARG;
  if (!h->have_grid) return SCF_ERR_STATE;
  CK(cudaSetDevice(h->device));
  const int nx = h->nx, ny = h->ny;
  const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2);
  int rc;
  if (!h->geo_alloc) {
    struct { void** p; size_t bytes; } a[] = {
        {(void**)&h->g_aE, n0 * 8}, {(void**)&h->g_aW, n0 * 8}, {(void**)&h->g_aN, n0 * 8},
        {(void**)&h->g_aS, n0 * 8}, {(void**)&h->g_WlLh, n1 * 8}, {(void**)&h->g_vofS, n1 * 8},
        {(void**)&h->g_nxS, n1 * 8}, {(void**)&h->g_nyS, n1 * 8}, {(void**)&h->g_vsu, n1 * 8},
        {(void**)&h->g_vsv, n1 * 8}, {(void**)&h->g_pp, n0 * 4}, {(void**)&h->g_pu, n0 * 4},
        {(void**)&h->g_pv, n0 * 4}, {(void**)&h->g_mu, n1 * 4}, {(void**)&h->g_mv, n1 * 4},
        {(void**)&h->g_st0, n0}, {(void**)&h->g_st1, n0},
        {(void**)&h->g_counts, geometry_count_ints(nx) * 4}, {(void**)&h->g_flag, 4}};
    for (auto& e : a)
      if ((rc = dev_alloc(h, e.p, e.bytes))) return rc;
    if (!h->devptrs)
      for (int k = 0; k < 6; ++k)
        if ((rc = dev_alloc(h, (void**)&h->g_in[k], n1 * 8))) return rc;
    if (cudaMallocHost((void**)&h->g_flag_host, sizeof(int)) != cudaSuccess) return SCF_ERR_NOMEM;
    h->geo_alloc = true;
  }
  if ((rc = put(h, &h->st_vof, vof, n1)) || (rc = put(h, &h->st_phi, phi, n1))) return rc;
  const double* src[6] = {vofS, phiS, nxS, nyS, vofS_u, vofS_v};
  const double* dev[6];
  for (int k = 0; k < 6; ++k) {
    if (h->devptrs) {
      dev[k] = src[k];
    } else {
      CK(cudaMemcpyAsync(h->g_in[k], src[k], n1 * 8, cudaMemcpyHostToDevice, h->stream));
      dev[k] = h->g_in[k];
    }
  }
  GeoIn gi{nx, ny, h->fin.dx, h->fin.dy, dev[0], dev[1], dev[2], dev[3], dev[4], dev[5]};
  GeoOut go{h->fin.dx, h->fin.dy, h->g_aE, h->g_aW, h->g_aN, h->g_aS, h->g_WlLh, h->g_vofS,
            h->g_nxS, h->g_nyS, h->g_vsu, h->g_vsv, h->g_pp, h->g_pu, h->g_pv, h->g_mu, h->g_mv};
  const int sweeps = geometry_build(gi, go, h->g_st0, h->g_st1, h->g_counts, h->g_flag,
                                    h->g_flag_host, icorprob ? 1 : 0, h->stream);
  if (sweeps < 0) {
    (void)cudaGetLastError();
    return SCF_ERR_CUDA;
  }
  h->geo_sweeps = sweeps;
  FortranIn& f = h->fin;
  f.vof = h->st_vof; f.phi = h->st_phi; f.vofS = h->g_vofS; f.nyS = h->g_nyS;
  f.WlLh = h->g_WlLh; f.aE = h->g_aE; f.aW = h->g_aW; f.aN = h->g_aN; f.aS = h->g_aS;
  f.posnu_p = h->g_pp; f.posnu_u = h->g_pu; f.posnu_v = h->g_pv;
  f.moex_u = h->g_mu; f.moex_v = h->g_mv; f.vofS_u = h->g_vsu; f.vofS_v = h->g_vsv;
  CK(cudaStreamSynchronize(h->stream));
  h->late_pending = false;  // the U/V arrays now come from the GPU geometry
  h->have_geom = true;
  h->assembled = false;
  return SCF_OK;
}

int scf_proj_get_geometry(scf_proj* h, double* vofS, double* nxS, double* nyS, double* WlLh,
                          double* aE, double* aW, double* aN, double* aS, int32_t* posnu_p,
                          int32_t* posnu_u, int32_t* posnu_v, int32_t* moex_u,
                          int32_t* moex_v, double* vofS_u, double* vofS_v) {
  if (!h) return SCF_ERR_ARG;
  if (!h->have_geom) return SCF_ERR_STATE;
  CK(cudaSetDevice(h->device));
  if (h->late_pending) {  // U/V arrays not copied yet: copy them now
    for (const auto& e : h->late)
      CK(cudaMemcpyAsync(e.dst, e.src, e.bytes, cudaMemcpyHostToDevice, h->stream));
    h->late_pending = false;
  }
  const FortranIn& f = h->fin;
  const size_t n1 = (size_t)h->nx * h->ny, n0 = (size_t)(h->nx + 2) * (h->ny + 2);
  const bool own = f.vofS == h->g_vofS && h->geo_alloc;
  if (nxS && !own) return SCF_ERR_STATE;
  struct { void* dst; const void* src; size_t bytes; } c[] = {
      {vofS, f.vofS, n1 * 8}, {nxS, own ? h->g_nxS : nullptr, n1 * 8}, {nyS, f.nyS, n1 * 8},
      {WlLh, f.WlLh, n1 * 8}, {aE, f.aE, n0 * 8}, {aW, f.aW, n0 * 8}, {aN, f.aN, n0 * 8},
      {aS, f.aS, n0 * 8}, {posnu_p, f.posnu_p, n0 * 4}, {posnu_u, f.posnu_u, n0 * 4},
      {posnu_v, f.posnu_v, n0 * 4}, {moex_u, f.moex_u, n1 * 4}, {moex_v, f.moex_v, n1 * 4},
      {vofS_u, f.vofS_u, n1 * 8}, {vofS_v, f.vofS_v, n1 * 8}};
  for (auto& e : c)
    if (e.dst && e.src)
      CK(cudaMemcpyAsync(e.dst, e.src, e.bytes, cudaMemcpyDefault, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return SCF_OK;
}

int scf_proj_get_operator(scf_proj* h, double* cE, double* cN, double* diag, double* rhs) {
  if (!h) return SCF_ERR_ARG;
  if (!h->assembled) return SCF_ERR_STATE;
  CK(cudaSetDevice(h->device));
  const size_t n1 = (size_t)h->nx * h->ny;
  double* tmp = nullptr;
  CK(cudaMallocAsync((void**)&tmp, n1 * 8, h->stream));
  const double* srcs[4] = {h->lev[0].cE, h->lev[0].cN, h->lev[0].dg, h->bvec};
  double* dsts[4] = {cE, cN, diag, rhs};
  int rc = SCF_OK;
  for (int a = 0; a < 4 && rc == SCF_OK; ++a) {
    if (!dsts[a]) continue;
    launch_to_fortran(h->lev[0], srcs[a], tmp, h->stream);
    if (cudaMemcpyAsync(dsts[a], tmp, n1 * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
      rc = SCF_ERR_CUDA;
  }
  cudaFreeAsync(tmp, h->stream);
  CK(cudaStreamSynchronize(h->stream));
  return rc;
}

int scf_diag_tma_timeout(int device, int cta, int spins) {
  if (cta < -1 || spins < 1) return SCF_ERR_ARG;
  CK(cudaSetDevice(device));
  CK(cudaDeviceSynchronize());  // no sweep of an earlier call sees a half-set pair
  return set_tma_fault(cta, spins) == 0 ? SCF_OK : SCF_ERR_CUDA;
}

int scf_proj_get_matrix(scf_proj* h, double* matr, int* asym_faces, double* asym_max) {
  if (!h) return SCF_ERR_ARG;
  if (!h->assembled) return SCF_ERR_STATE;
  CK(cudaSetDevice(h->device));
  const size_t n1 = (size_t)h->nx * h->ny;
  int rc = SCF_OK;
  if (matr) {
    double* tmp = nullptr;
    CK(cudaMallocAsync((void**)&tmp, 5 * n1 * 8, h->stream));
    launch_matr_out(h->fin, h->lev[0], tmp, h->stream);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(matr, tmp, 5 * n1 * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
      rc = SCF_ERR_CUDA;
    cudaFreeAsync(tmp, h->stream);
  }
  if (rc == SCF_OK)
    CK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (rc == SCF_OK) {
    if (asym_faces) *asym_faces = h->sc_host->asym_faces;
    if (asym_max) {
      unsigned b = h->sc_host->asym_max_bits;
      float f;
      memcpy(&f, &b, sizeof(f));
      *asym_max = (double)f;
    }
  }
  return rc;
}

int scf_proj_time_kernel(scf_proj* h, int kernel, int reps, double* ms) {
  if (!h || !ms || reps < 1 || kernel < 0 || kernel > SCF_K_FINE_POST) return SCF_ERR_ARG;
  if (!h->assembled) return SCF_ERR_STATE;
  CK(cudaSetDevice(h->device));
  cudaStream_t s = h->stream;
  // diagnostic scalars that never signal convergence
  Scalars init;
  memset(&init, 0, sizeof(init));
  init.maxit = 0x7fffffff;
  init.rtol2 = -1.0;
  CK(cudaMemcpyAsync(h->sc_diag, &init, sizeof(init), cudaMemcpyHostToDevice, s));
  LevelView L0 = h->lev[0];
  const bool two = h->lev.size() > 1;
  const double om = h->opts.omega;
  cudaGraphExec_t vexec = nullptr;
  if (kernel == SCF_K_VCYCLE) {  // one V-cycle as a graph, replayed
    cudaStream_t cs = nullptr;
    CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
    enqueue_vcycle(h, h->sc_diag, false, cs);
    CK(cudaStreamEndCapture(cs, &g));
    CK(cudaGraphInstantiate(&vexec, g, 0));
    cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
  }
  auto launch = [&]() {
    if (kernel == SCF_K_VCYCLE) {
      cudaGraphLaunch(vexec, s);
      return;
    }
    if (kernel == SCF_K_SETUP) {
      enqueue_setup(h, h->sc_diag, s);
      return;
    }
    if (kernel == SCF_K_PUPDATE_SPMV) {
      if (h->mixed)
        launch_pupdate_spmv_t<float>(L0, buf32(h, 0, 0), reinterpret_cast<const float*>(h->pA),
                                     reinterpret_cast<float*>(h->pB), h->q, h->sc_diag, h->part, s);
      else
        launch_pupdate_spmv_t<double>(L0, L0.x, h->pA, h->pB, h->q, h->sc_diag, h->part, s);
      return;
    }
    if (kernel == SCF_K_UPDATE_XR) {
      if (h->mixed)
        launch_update_xr(L0, h->xsol, reinterpret_cast<const float*>(h->pB), L0.b, h->r32,
                         buf32(h, 0, 0), h->q, h->sc_diag, h->part, 0ull, s);
      else
        launch_update_xr(L0, h->xsol, h->pB, L0.b, h->r32, nullptr, h->q, h->sc_diag, h->part,
                         0ull, s);
      return;
    }
    if (kernel == SCF_K_ASSEMBLE) {
      launch_assemble(h->fin, L0, h->sc_diag, s);
      return;
    }
    if (kernel == SCF_K_LINE) {  // one fine-level pass along x, as the V-cycle runs it
      if (h->mixed) {
        MgF V = h->mix[0];
        V.b = h->r32;
        launch_line(V, 1, false, h->sc_diag, s);
      } else if (!h->lf64n.empty()) {
        launch_line_solve<double, double>(view64(h, 0), h->lf64n[0], 1, false, h->sc_diag, s);
      } else {
        launch_line(view64(h, 0), 1, false, h->sc_diag, s);
      }
      return;
    }
    if (!two) return;
    if (kernel == SCF_K_FINE_PRE || kernel == SCF_K_FINE_POST) {
      // the fine level's first pre-smoothing and last post-smoothing launches
      // of the point-smoothed V-cycle, with the handle's fused iteration count
      const bool pre = kernel == SCF_K_FINE_PRE;
      const std::vector<int> it = sweep_launches(pre ? h->opts.npre : h->opts.npost, h->mixed);
      const int iters = pre ? it.front() : it.back();
      const bool one = it.size() == 1;  // that launch is also the last (pre) / first (post)
      const bool zero = pre, restr = pre && one, prol = !pre && one, rz = !pre;
      if (h->mixed) {
        MgF V = h->mix[0];
        V.b = h->r32;
        V.xin = pre ? nullptr : buf32(h, 0, 0);
        V.x = buf32(h, 0, 1);
        if (tma_level(h, 0))
          launch_sweep_tma(V, h->mix[1], h->dmaps[0], 0, pre ? 0 : 1, zero, prol, restr, rz, om,
                           1, h->sc_diag, h->part, s, iters);
        else
          launch_sweep(V, h->mix[1], pre ? 0 : 1, zero, prol, restr, rz, om, 1, h->sc_diag,
                       h->part, s, iters, h->tile);
      } else {
        MgD V = view64(h, 0);
        V.xin = pre ? nullptr : buf64(h, 0, 0);
        V.x = buf64(h, 0, 1);
        launch_sweep(V, view64(h, 1), pre ? 0 : 1, zero, prol, restr, rz, om, 0, h->sc_diag,
                     h->part, s, iters, h->tile);
      }
      return;
    }
    const bool smooth = kernel == SCF_K_SMOOTH, restr = kernel == SCF_K_RESID_RESTRICT,
               prol = kernel == SCF_K_PROLONG;
    const int first = restr ? 0 : 1;
    if (!h->mixed) {
      MgD V = view64(h, 0);
      V.xin = buf64(h, 0, 0);
      V.x = buf64(h, 0, 1);
      launch_sweep(V, view64(h, 1), first, false, prol, restr, false, om, 0, h->sc_diag, h->part,
                   s);
    } else {
      MgF V = h->mix[0];
      V.xin = buf32(h, 0, 0);
      V.x = buf32(h, 0, 1);
      V.b = h->r32;
      if (tma_level(h, 0))
        launch_sweep_tma(V, h->mix[1], h->dmaps[0], 0, first, false, prol, restr, false, om, 1,
                         h->sc_diag, h->part, s, 1);
      else
        launch_sweep(V, h->mix[1], first, false, prol, restr, false, om, 1, h->sc_diag, h->part,
                     s);
    }
    (void)smooth;
  };
  launch();  // warm-up
  CK(cudaEventRecord(h->ev[5], s));
  for (int r = 0; r < reps; ++r) launch();
  CK(cudaEventRecord(h->ev[6], s));
  // the assembly alone clears the row flags of the exact west / south
  // entries; the excess pass raises them again (same operator, same bits)
  if (kernel == SCF_K_ASSEMBLE)
    launch_excess(L0, h->mixed ? nullptr : h->di64[0], nullptr, 0, h->sc_diag, s);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  if (vexec) cudaGraphExecDestroy(vexec);
  *ms = (double)elapsed(h->ev[5], h->ev[6]) / reps;
  return SCF_OK;
}

struct scf_batch {
  std::vector<scf_proj*> h;
  std::vector<BatchIO> io;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  float last_ms = 0.0f;
  std::vector<long long> once, body;  // kernel nodes per branch: outside / inside the loop
};

int scf_batch_create(scf_batch** out, scf_proj* const* handles, int count) {
  if (!out || !handles || count < 1) return SCF_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < count; ++i) {
    scf_proj* h = handles[i];
    if (!h || !h->devptrs || h->device != handles[0]->device || learned(h) ||
        (h->opts.flags & SCF_FLAG_NO_GRAPH))
      return SCF_ERR_ARG;
    if (!h->assembled) return SCF_ERR_STATE;
    for (int j = 0; j < i; ++j)
      if (handles[j] == h) return SCF_ERR_ARG;
  }
  scf_batch* b = new (std::nothrow) scf_batch();
  if (!b) return SCF_ERR_NOMEM;
  b->h.assign(handles, handles + count);
  b->io.resize(count);
  CK(cudaSetDevice(handles[0]->device));
  if (cudaEventCreate(&b->ev[0]) != cudaSuccess || cudaEventCreate(&b->ev[1]) != cudaSuccess) {
    delete b;
    return SCF_ERR_CUDA;
  }
  *out = b;
  return SCF_OK;
}

int scf_batch_destroy(scf_batch* b) {
  if (!b) return SCF_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto e : b->ev)
    if (e) cudaEventDestroy(e);
  delete b;
  return SCF_OK;
}

int scf_batch_set_io(scf_batch* b, int i, const double* ustar, const double* vstar, double vb,
                     double* Pp, double* p, double* u, double* v, double* mres) {
  if (!b || i < 0 || i >= (int)b->h.size() || !ustar || !vstar || !Pp || !p || !u || !v || !mres)
    return SCF_ERR_ARG;
  BatchIO& io = b->io[i];
  io.ustar = ustar; io.vstar = vstar; io.vb = vb;
  io.Pp = Pp; io.p = p; io.u = u; io.v = v; io.mres = mres;
  io.set = true;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  return SCF_OK;
}

int scf_batch_run(scf_batch* b, void* stream, scf_stats* stats) {
  if (!b) return SCF_ERR_ARG;
  for (const BatchIO& io : b->io)
    if (!io.set) return SCF_ERR_STATE;
  for (scf_proj* h : b->h)
    if (!h->assembled) return SCF_ERR_STATE;
  CK(cudaSetDevice(b->h[0]->device));
  cudaStream_t s = (cudaStream_t)stream;
  if (!b->exec) {
    CK(cudaDeviceSynchronize());
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    cudaStream_t cs = nullptr, cs2 = nullptr;
    CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&cs2, cudaStreamNonBlocking));
    int rc = SCF_OK;
    b->once.assign(b->h.size(), 0);
    b->body.assign(b->h.size(), 0);
    for (size_t i = 0; i < b->h.size() && rc == SCF_OK; ++i)
      rc = add_batch_branch(b->h[i], b->io[i], g, cs, cs2, &b->once[i], &b->body[i]);
    cudaStreamDestroy(cs);
    cudaStreamDestroy(cs2);
    if (rc == SCF_OK && cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) rc = SCF_ERR_CUDA;
    if (rc != SCF_OK) {
      cudaGetLastError();
      cudaGraphDestroy(g);
      b->exec = nullptr;
      return rc;
    }
    b->graph = g;
  }
  CK(cudaEventRecord(b->ev[0], s));
  CK(cudaGraphLaunch(b->exec, s));
  CK(cudaEventRecord(b->ev[1], s));
  CK(cudaStreamSynchronize(s));
  b->last_ms = elapsed(b->ev[0], b->ev[1]);
  int worst = SCF_OK;
  for (size_t i = 0; i < b->h.size(); ++i) {
    const Scalars& S = *b->h[i]->sc_host;
    int status = (S.nan || S.anan) ? SCF_ERR_NAN : S.status;
    if (status != kOk && worst == SCF_OK) worst = status;
    if (stats) {
      scf_stats& st = stats[i];
      memset(&st, 0, sizeof(st));
      st.iters = S.iter;
      st.status = status;
      st.levels = (int)b->h[i]->lev.size();
      st.smoother = b->h[i]->line ? SCF_SMOOTH_LINE : SCF_SMOOTH_POINT;
      st.bnorm = sqrt(S.bnorm2);
      st.relres = S.bnorm2 > 0 ? sqrt(S.rr / S.bnorm2) : 0.0;
      st.relres_true = S.bnorm2 > 0 ? sqrt(S.res_true2 / S.bnorm2) : 0.0;
      st.mres_max = S.mres_max;
      st.ms_total = b->last_ms;
      st.launches = (int)(b->once[i] + (long long)(S.pad[0] / 2) * b->body[i]);
    }
  }
  return worst;
}

int scf_proj_set_opts(scf_proj* h, int npre, int npost, double omega) {
  if (!h || npre < 1 || npost < 1 || npre > 8 || npost > 8 || !(omega > 0.0 && omega < 2.0))
    return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  h->opts.npre = npre;
  h->opts.npost = npost;
  h->opts.omega = omega;
  // the tails carry their own copy of the schedule
  h->tail64.npre = h->tail32.npre = h->ltail64.npre = h->ltail32.npre = npre;
  h->tail64.npost = h->tail32.npost = h->ltail64.npost = h->ltail32.npost = npost;
  h->tail64.omega = omega;
  h->tail32.omega = (float)omega;
  h->ltail64.omega = omega;
  h->ltail32.omega = (float)omega;
  destroy_graph(h);
  if (h->assembled && !(h->opts.flags & SCF_FLAG_NO_GRAPH)) return build_graph(h);
  return SCF_OK;
}

int scf_proj_set_coarse_sweeps(scf_proj* h, int coarse_from, int sweeps) {
  if (!h || sweeps < 0 || sweeps > 8 || coarse_from < 0 || coarse_from > 64) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  h->opts.coarse_sweeps = sweeps;
  h->opts.coarse_from = coarse_from;
  // the tails carry their own copy of the schedule
  if (h->tail0 > 0) {
    set_tail_coarse(h->tail64, h->opts, h->tail0);
    set_tail_coarse(h->tail32, h->opts, h->tail0);
  }
  if (h->ltail0 > 0) {
    set_tail_coarse(h->ltail64, h->opts, h->ltail0);
    set_tail_coarse(h->ltail32, h->opts, h->ltail0);
  }
  destroy_graph(h);
  if (h->assembled && !(h->opts.flags & SCF_FLAG_NO_GRAPH)) return build_graph(h);
  return SCF_OK;
}

int scf_proj_set_tile(scf_proj* h, int tile) {
  if (!h || (tile != SCF_TILE_64X32 && tile != SCF_TILE_32X32)) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  if (tile == h->tile) return SCF_OK;
  h->tile = tile;
  destroy_graph(h);
  if (h->assembled && !(h->opts.flags & SCF_FLAG_NO_GRAPH)) return build_graph(h);
  return SCF_OK;
}

int scf_proj_set_network(scf_proj* h, const float* params, int nparams) {
  if (!h || !params || nparams != UNet::num_params()) return SCF_ERR_ARG;
  if (!h->mixed) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  if (!h->net) {
    UNet* u = new (std::nothrow) UNet();
    if (!u) return SCF_ERR_NOMEM;
    const int H = (h->ny + 7) / 8 * 8, W = (h->nx + 7) / 8 * 8;
    if (u->create(1, H, W, false, h->device) != 0) {
      delete u;
      return SCF_ERR_NOMEM;
    }
    h->net = u;
    int rc;
    if (!h->net_sigma && (rc = dev_alloc(h, (void**)&h->net_sigma, sizeof(float)))) return rc;
  }
  if (h->net->set_params_host(params) != 0) return SCF_ERR_CUDA;
  return SCF_OK;
}

int scf_proj_solve_rhs(scf_proj* h, const double* b, double* x, double* r, int maxit,
                       scf_stats* st) {
  if (!h || !b || !x) return SCF_ERR_ARG;
  if (!h->assembled) return SCF_ERR_STATE;
  if (maxit < 0 || maxit > h->opts.maxit) return SCF_ERR_ARG;
  if (learned(h) && !h->net) return SCF_ERR_STATE;
  CK(cudaSetDevice(h->device));
  cudaStream_t s = h->stream;
  const size_t n1 = (size_t)h->nx * h->ny;
  const double* db = b;
  double *dx = x, *dr = r;
  if (!h->devptrs) {  // the (nx+2)(ny+2) velocity staging buffers hold (nx,ny) arrays
    CK(cudaMemcpyAsync(h->st_us, b, n1 * 8, cudaMemcpyHostToDevice, s));
    db = h->st_us;
    dx = h->st_vs;
    dr = r ? h->st_Pp : nullptr;
  }
  CK(cudaEventRecord(h->ev[1], s));
  const long long l0 = g_launches;
  h->body_runs = 0;
  LevelView L0 = h->lev[0];
  CK(cudaMemsetAsync(&h->sc->nan, 0, sizeof(int), s));
  launch_rhs_given(h->nx, h->ny, db, L0, h->bvec, L0.b, h->r32, h->xsol, h->sc, h->part,
                   h->opts.rtol, maxit, s);
  CK(cudaGetLastError());
  int nn_iters = 0, fell_back = 0, rc = SCF_OK;
  if (maxit > 0) {
    const int saved = h->opts.maxit;
    h->opts.maxit = maxit;  // bound of the host-polled loops
    rc = learned(h) ? run_learned(h, &nn_iters, &fell_back) : run_pcg(h);
    h->opts.maxit = saved;
    if (rc) return rc;
  }
  CK(cudaEventRecord(h->ev[2], s));
  launch_final_solution(h->fin, L0, h->xsol, h->bvec, nullptr, nullptr, nullptr, nullptr,
                        nullptr, nullptr, 0, h->sc, h->part, s);
  launch_to_fortran(L0, h->xsol, dx, s);
  if (dr) launch_to_fortran(L0, L0.b, dr, s);
  CK(cudaGetLastError());
  if (!h->devptrs) {
    CK(cudaMemcpyAsync(x, dx, n1 * 8, cudaMemcpyDeviceToHost, s));
    if (r) CK(cudaMemcpyAsync(r, dr, n1 * 8, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const Scalars& S = *h->sc_host;
  int status = S.status;
  if (S.nan || S.anan) status = SCF_ERR_NAN;
  if (maxit == 0 && S.bnorm2 > 0) status = SCF_ERR_NOT_CONVERGED;
  if (st) {
    memset(st, 0, sizeof(*st));
    st->iters = S.iter;
    st->status = status;
    st->levels = (int)h->lev.size();
    st->fallbacks = fell_back;
    st->learned_iters = nn_iters;
    st->smoother = h->line ? SCF_SMOOTH_LINE : SCF_SMOOTH_POINT;
    st->bnorm = sqrt(S.bnorm2);
    st->relres = S.bnorm2 > 0 ? sqrt(S.rr / S.bnorm2) : 0.0;
    st->relres_true = S.bnorm2 > 0 ? sqrt(S.res_true2 / S.bnorm2) : 0.0;
    st->ms_solve = elapsed(h->ev[1], h->ev[2]);
    long long n = h->pending_launches + (g_launches - l0);
    if (maxit > 0 && h->graph_cond && h->gexec && !learned(h))
      n += (long long)(S.pad[0] / 2) * h->body_launches;
    n += h->body_runs * h->body_launches;
    st->launches = (int)n;
    st->asym_faces = S.asym_faces;
  }
  h->pending_launches = 0;
  return status == kOk ? SCF_OK : status;
}

int scf_proj_vcycle(scf_proj* h, const double* b, double* x) {
  if (!h || !b || !x) return SCF_ERR_ARG;
  if (!h->assembled) return SCF_ERR_STATE;
  CK(cudaSetDevice(h->device));
  const size_t n1 = (size_t)h->nx * h->ny;
  double* tmp = nullptr;
  cudaStream_t s = h->stream;
  CK(cudaMallocAsync((void**)&tmp, n1 * 8, s));
  CK(cudaMemcpyAsync(tmp, b, n1 * 8, cudaMemcpyHostToDevice, s));
  launch_from_fortran(h->lev[0], tmp, h->lev[0].b, s);
  if (h->mixed) launch_from_fortran_f(h->lev[0], tmp, h->r32, s);
  CK(cudaMemsetAsync(h->sc_diag, 0, sizeof(Scalars), s));
  enqueue_vcycle(h, h->sc_diag, false, s);
  const int zf = final_buf(h, 0);
  if (h->mixed) launch_to_fortran_f(h->lev[0], buf32(h, 0, zf), tmp, s);
  else launch_to_fortran(h->lev[0], buf64(h, 0, zf), tmp, s);
  CK(cudaMemcpyAsync(x, tmp, n1 * 8, cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(tmp, s);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  return SCF_OK;
}

}  // extern "C"

namespace scf {

int mgpre_create(scf_proj** out, int nx, int ny, int device) {
  scf_opts o;
  scf_opts_default(&o);
  o.precision = SCF_PREC_FP64;
  o.smoother = SCF_SMOOTH_POINT;
  o.flags = SCF_FLAG_DEVICE_PTRS | SCF_FLAG_NO_GRAPH;
  o.device = device;
  o.npre = 2;
  o.npost = 2;
  // aggregation's coarse operator is too stiff for smooth errors, as for the
  // pressure (measured on the 2048^2 u solve at Re 0.01: 111 BiCGStab
  // iterations at omega 1.0, 26 at 1.5, 19 at 1.8, 17 at 1.9; 4 at every
  // omega at Re 1e5)
  o.omega = 1.9;
  return scf_proj_create(out, nx, ny, &o);
}

int mgpre_setup(scf_proj* h, const double* P, const double* W, const double* E,
                const double* S, const double* N, cudaStream_t s) {
  if (!h || !P || !W || !E || !S || !N) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  const LevelView& L0 = h->lev[0];
  launch_k(k_mgpre_level0, grid_for(L0.nx, L0.ny, 1), dim3(32, 8), 0, s, L0, P, W, E, S, N);
  CK(cudaMemsetAsync(h->sc_diag, 0, sizeof(Scalars), s));
  enqueue_setup_levels(h, h->sc_diag, s);
  CK(cudaGetLastError());
  h->assembled = true;
  return SCF_OK;
}

int mgpre_apply(scf_proj* h, double* b, double* z, cudaStream_t s) {
  if (!h || !b || !z || !h->assembled || h->mixed || h->line) return SCF_ERR_STATE;
  // the V-cycle reads level 0's b and ends in level 0's final buffer: both
  // are pointed at the caller's arrays for the duration of the enqueue (the
  // launches take the views by value)
  const int zf = final_buf(h, 0);
  double* const b0 = h->lev[0].b;
  double** xf = zf == 0 ? &h->lev[0].x : &h->x2_64[0];
  double* const x0 = *xf;
  h->lev[0].b = b;
  *xf = z;
  CK(cudaMemsetAsync(h->sc_diag, 0, sizeof(Scalars), s));
  enqueue_vcycle(h, h->sc_diag, false, s);
  h->lev[0].b = b0;
  *xf = x0;
  CK(cudaGetLastError());
  return SCF_OK;
}

}  // namespace scf
