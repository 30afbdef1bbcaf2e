// scf_proj.cu -- host side of libscf_proj.so: the C-ABI declared in
// include/scf_proj.h.  Owns the device memory, the multigrid hierarchy and
// the CUDA graph of the PCG loop.
//
// The PCG loop runs entirely on the device: one CUDA graph holds a
// conditional WHILE node whose body is two PCG iterations (the direction
// vector ping-pongs between two buffers); the convergence test in the last
// kernel of each iteration clears the loop condition.  No host round trip
// happens between the right-hand side and the final correction.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/scf_proj.h"
#include "scf_internal.cuh"

using namespace scf;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct scf_proj {
  int nx = 0, ny = 0;
  scf_opts opts;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool devptrs = false;

  // multigrid levels (level 0 is the fine grid; its b is the PCG residual r
  // and its x the preconditioned residual z)
  std::vector<LevelView> lev;
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
  double *st_us = nullptr, *st_vs = nullptr, *st_Pp = nullptr, *st_p = nullptr, *st_u = nullptr,
         *st_v = nullptr, *st_mres = nullptr;

  bool have_grid = false, have_geom = false, assembled = false;

  // graph of the PCG loop
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graph_cond = false;     // true: conditional while-node graph
  cudaGraph_t body_graph = nullptr;
  cudaGraphExec_t body_exec = nullptr;  // fallback: body only, host-polled

  cudaEvent_t ev[8];
};

namespace {

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      if (getenv("SCF_DEBUG")) fprintf(stderr, "scf: %s failed: %s (%s:%d)\n", #call, \
                                       cudaGetErrorString(e_), __FILE__, __LINE__); \
      return e_ == cudaErrorMemoryAllocation ? SCF_ERR_NOMEM : SCF_ERR_CUDA;       \
    }                                                                              \
  } while (0)

int dev_alloc(scf_proj* h, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? SCF_ERR_NOMEM : SCF_ERR_CUDA;
  h->allocs.push_back(*p);
  e = cudaMemsetAsync(*p, 0, bytes ? bytes : 16, h->stream);
  return e == cudaSuccess ? SCF_OK : SCF_ERR_CUDA;
}

// padded array for a level: (ny+3)*pitch elements, base at row 2
int level_array(scf_proj* h, int ny, int pitch, double** base) {
  void* p = nullptr;
  size_t n = (size_t)(ny + 3) * pitch;
  int rc = dev_alloc(h, &p, n * sizeof(double));
  if (rc) return rc;
  *base = reinterpret_cast<double*>(p) + 2 * (size_t)pitch;
  return SCF_OK;
}

void fill_fin(scf_proj* h) {
  FortranIn& f = h->fin;
  f.nx = h->nx; f.ny = h->ny;
}

void destroy_graph(scf_proj* h) {
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->graph) cudaGraphDestroy(h->graph);
  if (h->body_exec) cudaGraphExecDestroy(h->body_exec);
  if (h->body_graph) cudaGraphDestroy(h->body_graph);
  h->gexec = nullptr; h->graph = nullptr; h->body_exec = nullptr; h->body_graph = nullptr;
}

// Enqueue one multigrid V-cycle on level 0 (b -> x).  do_rz: the last
// kernel also reduces r.z and sets the PCG beta.
void enqueue_vcycle(scf_proj* h, Scalars* sc, bool do_rz, cudaStream_t s) {
  const int L = (int)h->lev.size();
  const int npre = h->opts.npre, npost = h->opts.npost;
  if (L == 1) {
    launch_coarse_solve(h->lev[0], h->Ainv, h->cmap, h->ncoarse, sc, s);
    if (do_rz) launch_dot_rz(h->lev[0], sc, h->part, s);
    return;
  }
  for (int l = 0; l < L - 1; ++l) {
    for (int it = 0; it < npre; ++it) {
      launch_smooth(h->lev[l], 0, it == 0 ? 1 : 0, 0, sc, h->part, s);
      launch_smooth(h->lev[l], 1, 0, 0, sc, h->part, s);
    }
    if (npre == 0) {
      // iterate starts at zero without a smoothing sweep
      cudaMemsetAsync(h->lev[l].x - 2 * (size_t)h->lev[l].pitch, 0,
                      sizeof(double) * (size_t)(h->lev[l].ny + 3) * h->lev[l].pitch, s);
    }
    launch_resid_restrict(h->lev[l], h->lev[l + 1], sc, s);
  }
  launch_coarse_solve(h->lev[L - 1], h->Ainv, h->cmap, h->ncoarse, sc, s);
  for (int l = L - 2; l >= 0; --l) {
    launch_prolong(h->lev[l], h->lev[l + 1], h->opts.omega, sc, s);
    for (int it = 0; it < npost; ++it) {
      bool last = (l == 0 && it == npost - 1);
      launch_smooth(h->lev[l], 1, 0, 0, sc, h->part, s);
      launch_smooth(h->lev[l], 0, 0, (last && do_rz) ? 1 : 0, sc, h->part, s);
    }
  }
  if (npost == 0 && do_rz) launch_dot_rz(h->lev[0], sc, h->part, s);
}

// one PCG iteration: z = M r, beta, p = z + beta p_old, q = A p, alpha,
// x += alpha p, r -= alpha q, convergence test
void enqueue_iteration(scf_proj* h, const double* pold, double* pnew, unsigned long long cond,
                       cudaStream_t s) {
  LevelView L0 = h->lev[0];
  enqueue_vcycle(h, h->sc, true, s);
  launch_pupdate_spmv(L0, L0.x, pold, pnew, h->q, h->sc, h->part, s);
  launch_update_xr(L0, h->xsol, pnew, L0.b, h->q, h->sc, h->part, cond, s);
}

int build_graph(scf_proj* h) {
  destroy_graph(h);
  if (h->opts.flags & SCF_FLAG_NO_GRAPH) return SCF_OK;
  cudaStream_t cs = nullptr;
  CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  // preferred: conditional while node
  bool ok = false;
  do {
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
    enqueue_iteration(h, h->pA, h->pB, (unsigned long long)handle, cs);
    enqueue_iteration(h, h->pB, h->pA, (unsigned long long)handle, cs);
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &captured);
    if (e != cudaSuccess) {
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
  if (!ok) {
    // fallback: graph of the loop body, relaunched and polled from the host
    cudaGetLastError();
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
    enqueue_iteration(h, h->pA, h->pB, 0ull, cs);
    enqueue_iteration(h, h->pB, h->pA, 0ull, cs);
    CK(cudaStreamEndCapture(cs, &h->body_graph));
    CK(cudaGraphInstantiate(&h->body_exec, h->body_graph, 0));
    h->graph_cond = false;
  }
  cudaStreamDestroy(cs);
  return SCF_OK;
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
      } else {
        enqueue_iteration(h, h->pA, h->pB, 0ull, h->stream);
        enqueue_iteration(h, h->pB, h->pA, 0ull, h->stream);
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

int solve_common(scf_proj* h, const double* ustar, const double* vstar, double vb, double* Pp,
                 double* p, double* u, double* v, double* mres, scf_stats* st, bool correct) {
  if (!h) return SCF_ERR_ARG;
  if (!h->assembled) return SCF_ERR_STATE;
  if (!ustar || !vstar) return SCF_ERR_ARG;
  if (correct && (!p || !u || !v || !mres)) return SCF_ERR_ARG;
  CK(cudaSetDevice(h->device));
  const int nx = h->nx, ny = h->ny;
  const size_t n0 = (size_t)(nx + 2) * (ny + 2), n1 = (size_t)nx * ny;
  cudaStream_t s = h->stream;
  CK(cudaEventRecord(h->ev[0], s));
  const double *dus = ustar, *dvs = vstar;
  double *dPp = Pp, *dp = p, *du = u, *dv = v, *dm = mres;
  if (!h->devptrs) {
    CK(cudaMemcpyAsync(h->st_us, ustar, n0 * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->st_vs, vstar, n0 * 8, cudaMemcpyHostToDevice, s));
    dus = h->st_us; dvs = h->st_vs;
    dPp = Pp ? h->st_Pp : nullptr;
    if (correct) {
      CK(cudaMemcpyAsync(h->st_p, p, n0 * 8, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(h->st_u, u, n0 * 8, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(h->st_v, v, n0 * 8, cudaMemcpyHostToDevice, s));
      dp = h->st_p; du = h->st_u; dv = h->st_v; dm = h->st_mres;
    }
  }
  CK(cudaEventRecord(h->ev[1], s));
  LevelView L0 = h->lev[0];
  // the NaN flag of a previous solve must not leak into this one
  CK(cudaMemsetAsync(&h->sc->nan, 0, sizeof(int), s));
  launch_rhs(h->fin, dus, dvs, vb, L0, h->bvec, L0.b, h->xsol, h->sc, h->part, h->opts.rtol,
             h->opts.maxit, s);
  CK(cudaGetLastError());
  int rc = run_pcg(h);
  if (rc) return rc;
  CK(cudaEventRecord(h->ev[2], s));
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
  if (S.nan) status = SCF_ERR_NAN;
  if (st) {
    st->iters = S.iter;
    st->status = status;
    st->levels = (int)h->lev.size();
    st->fallbacks = 0;
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
  }
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
  if (o.maxit < 1 || o.npre < 0 || o.npost < 0 || !(o.rtol >= 0.0)) return SCF_ERR_ARG;
  if (o.coarse_max < 1 || o.coarse_max > kMaxCoarse) return SCF_ERR_ARG;
  if (!(o.omega > 0.0 && o.omega < 2.0)) return SCF_ERR_ARG;
  scf_proj* h = new (std::nothrow) scf_proj();
  if (!h) return SCF_ERR_NOMEM;
  h->nx = nx; h->ny = ny; h->opts = o;
  h->device = o.device;
  h->devptrs = (o.flags & SCF_FLAG_DEVICE_PTRS) != 0;
  int rc = SCF_OK;
  auto fail = [&](int code) { scf_proj_destroy(h); return code; };
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(SCF_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(SCF_ERR_CUDA);
  h->own_stream = true;
  for (auto& e : h->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(SCF_ERR_CUDA);
  // multigrid levels
  int lx = nx, ly = ny;
  while (true) {
    LevelView L{};
    L.nx = lx; L.ny = ly; L.pitch = round_up(lx + 2, 32);
    double** arrs[6] = {&L.cE, &L.cN, &L.dg, &L.ex, &L.x, &L.b};
    for (auto a : arrs)
      if ((rc = level_array(h, ly, L.pitch, a))) return fail(rc);
    h->lev.push_back(L);
    if ((long)lx * ly <= o.coarse_max || (lx == 1 && ly == 1) || h->lev.size() >= 30) break;
    lx = (lx + 1) / 2; ly = (ly + 1) / 2;
  }
  const int P0 = h->lev[0].pitch;
  double** pv[5] = {&h->xsol, &h->pA, &h->pB, &h->q, &h->bvec};
  for (auto a : pv)
    if ((rc = level_array(h, ny, P0, a))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->Ainv, sizeof(double) * kMaxCoarse * kMaxCoarse))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->cmap, sizeof(int) * kMaxCoarse))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->ncoarse, sizeof(int)))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->sc, sizeof(Scalars)))) return fail(rc);
  if ((rc = dev_alloc(h, (void**)&h->sc_diag, sizeof(Scalars)))) return fail(rc);
  size_t nblk = 0;
  {
    dim3 g1 = grid_for(nx, ny, 1), g2 = grid_for(nx, ny, 2);
    nblk = (size_t)g1.x * g1.y;
    if ((size_t)g2.x * g2.y > nblk) nblk = (size_t)g2.x * g2.y;
  }
  if ((rc = dev_alloc(h, (void**)&h->part, sizeof(double) * (nblk + 32)))) return fail(rc);
  if (cudaMallocHost((void**)&h->sc_host, sizeof(Scalars)) != cudaSuccess) return fail(SCF_ERR_NOMEM);
  memset(h->sc_host, 0, sizeof(Scalars));
  // Fortran-layout staging (host mode only)
  if (!h->devptrs) {
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
  fill_fin(h);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(SCF_ERR_CUDA);
  *out = h;
  return SCF_OK;
}

int scf_proj_destroy(scf_proj* h) {
  if (!h) return SCF_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  destroy_graph(h);
  for (void* p : h->allocs) cudaFree(p);
  if (h->sc_host) cudaFreeHost(h->sc_host);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
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
      (rc = put(h, &h->st_aS, aS, n0)) || (rc = put(h, &h->st_pp, posnu_p, n0)) ||
      (rc = put(h, &h->st_pu, posnu_u, n0)) || (rc = put(h, &h->st_mu, moex_u, n1)) ||
      (rc = put(h, &h->st_vsu, vofS_u, n1)) || (rc = put(h, &h->st_pv, posnu_v, n0)) ||
      (rc = put(h, &h->st_mv, moex_v, n1)) || (rc = put(h, &h->st_vsv, vofS_v, n1)))
    return rc;
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
  CK(cudaMemsetAsync(h->sc, 0, sizeof(Scalars), s));
  launch_assemble(f, h->lev[0], h->sc, s);
  launch_excess(h->lev[0], s);
  for (size_t l = 1; l < h->lev.size(); ++l) launch_coarsen(h->lev[l - 1], h->lev[l], s);
  launch_coarse_setup(h->lev.back(), h->Ainv, h->cmap, h->ncoarse, s);
  CK(cudaGetLastError());
  int nanflag = 0;
  CK(cudaMemcpyAsync(&nanflag, &h->sc->nan, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (nanflag) return SCF_ERR_NAN;
  if (!h->gexec && !h->body_exec && !(h->opts.flags & SCF_FLAG_NO_GRAPH)) {
    if ((rc = build_graph(h))) return rc;
  }
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

int scf_proj_time_kernel(scf_proj* h, int kernel, int reps, double* ms) {
  if (!h || !ms || reps < 1 || kernel < 0 || kernel > SCF_K_ASSEMBLE) return SCF_ERR_ARG;
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
  auto launch = [&]() {
    switch (kernel) {
      case SCF_K_SMOOTH: launch_smooth(L0, 1, 0, 0, h->sc_diag, h->part, s); break;
      case SCF_K_PUPDATE_SPMV:
        launch_pupdate_spmv(L0, L0.x, h->pA, h->pB, h->q, h->sc_diag, h->part, s);
        break;
      case SCF_K_UPDATE_XR:
        launch_update_xr(L0, h->xsol, h->pB, L0.b, h->q, h->sc_diag, h->part, 0ull, s);
        break;
      case SCF_K_RESID_RESTRICT:
        if (h->lev.size() > 1) launch_resid_restrict(L0, h->lev[1], h->sc_diag, s);
        break;
      case SCF_K_PROLONG:
        if (h->lev.size() > 1) launch_prolong(L0, h->lev[1], h->opts.omega, h->sc_diag, s);
        break;
      case SCF_K_ASSEMBLE: launch_assemble(h->fin, L0, h->sc_diag, s); break;
    }
  };
  launch();  // warm-up
  CK(cudaEventRecord(h->ev[5], s));
  for (int r = 0; r < reps; ++r) launch();
  CK(cudaEventRecord(h->ev[6], s));
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  *ms = (double)elapsed(h->ev[5], h->ev[6]) / reps;
  return SCF_OK;
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
  CK(cudaMemsetAsync(h->sc_diag, 0, sizeof(Scalars), s));
  enqueue_vcycle(h, h->sc_diag, false, s);
  launch_to_fortran(h->lev[0], h->lev[0].x, tmp, s);
  CK(cudaMemcpyAsync(x, tmp, n1 * 8, cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(tmp, s);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  return SCF_OK;
}

}  // extern "C"
