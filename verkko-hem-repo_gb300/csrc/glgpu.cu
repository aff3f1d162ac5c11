// Context, C ABI entry points and the host-side control flow of the Newton path.
//
// Reference control flow restated here (paths relative to the reference root):
//   run()              femgl/src/run.cc:207-252   assemble -> solve -> newton_iteration -> test
//   assemble_system()  femgl/src/assemble.cc:109-372
//   compute_residual() femgl/src/residual.cc:110-297
//   solve(tol)         femgl/src/solve.cc:109-187 (FGMRES + ML AMG there; GMRES(m) with
//                      block-Jacobi or Chebyshev/block-Jacobi preconditioning here)
//   newton_iteration() femgl/src/iteration.cc:110-215
// All device work goes to the context's stream; the host only decides control flow
// from per-instance scalars (norms, flags) it reads back.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include <cuda_fp16.h>

#include "device.h"
#include "glgpu.h"
#include "glgpu_internal.h"

namespace glgpu
{
static thread_local std::string g_last_error;

glgpu_status set_error(glgpu_status s, const std::string &msg)
{
  g_last_error = msg;
  return s;
}

enum KernelKind
{
  KK_SPMV = 0,
  KK_CELL = 1,
  KK_ROWS = 2,
  KK_RES = 3,
  KK_PREC = 4,
  KK_VEC = 5,
  KK_N = 6
};

enum Phase
{
  PH_ASM = 0,
  PH_RES = 1,
  PH_SOLVE = 2,
  PH_NEWTON = 3,
  PH_N = 4
};

template <typename T> struct DBuf
{
  T *p = nullptr;
  size_t n = 0;
};

} // namespace glgpu

using namespace glgpu;

struct glgpu_ctx
{
  Plan P;
  DevMesh dm{};
  std::vector<glgpu_params> prm;
  // Kelly error estimator (built on first use): face pairs, per-cell lists, estimates
  struct Kelly
  {
    bool ready = false, eta_valid = false;
    int64_t np = 0;
    int32_t *a = nullptr, *b = nullptr, *cptr = nullptr, *cpair = nullptr;
    int8_t *fa = nullptr, *ob = nullptr, *sub = nullptr, *flags = nullptr;
    double *I = nullptr;
    float *eta = nullptr;
    uint32_t *prefix = nullptr, *hist = nullptr, *thr_r = nullptr, *thr_c = nullptr;
  } kelly;
  int B = 18, n_inst = 1, nq = 8, ns = 171;
  int64_t nn = 0, N = 0, nnzb = 0;
  bool mixed = false;
  int restart = 50;
  cudaStream_t st = nullptr;
  std::vector<void *> allocs;
  size_t dev_bytes = 0; // sum of this context's device allocations
  // state
  double *x = nullptr, *xt = nullptr, *delta = nullptr, *R = nullptr, *rhs = nullptr;
  double *r_cell = nullptr, *e_cell = nullptr;
  void *H = nullptr, *vals = nullptr, *dinv = nullptr;
  // Krylov (element type T = float in mixed mode, double otherwise)
  void *V = nullptr, *Z = nullptr, *X = nullptr, *Tmp = nullptr, *Bv = nullptr, *C1 = nullptr, *C2 = nullptr,
       *C3 = nullptr;
  double *partial = nullptr, *partial_n = nullptr;
  GmresDev g{};
  // per-instance small arrays (device)
  double *d_norm = nullptr, *d_a = nullptr, *d_energy = nullptr, *d_cheb = nullptr, *d_tmp = nullptr;
  uint8_t *d_act = nullptr, *d_act2 = nullptr;
  unsigned int *d_cnt = nullptr; // per-instance tickets of the in-kernel reductions
  // pinned host mirrors
  double *h_norm = nullptr, *h_res = nullptr;
  uint8_t *h_act = nullptr, *h_act_pipe = nullptr;
  int *h_its = nullptr;
  cudaEvent_t ev_pipe[2] = {nullptr, nullptr};
  // host-side per-instance state
  std::vector<double> rhs_norm, res_norm, lam_max;
  std::vector<uint8_t> inst_on;
  bool has_J = false, has_rhs = false, has_delta = false, prec_ready = false;
  // timing
  int ktiming = 0; // bitmask of kernel kinds timed with events
  int64_t launches = 0;
  int64_t klaunch[KK_N] = {0};
  double kms[KK_N] = {0};
  double phase_ms[PH_N] = {0};
  struct EvRec
  {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<EvRec> kev, pev;
  std::vector<cudaEvent_t> ev_pool;
  cudaEvent_t ev_user0 = nullptr, ev_user1 = nullptr;
  // multigrid (precond == GLGPU_PC_MULTIGRID on uniform box meshes)
  bool owns_stream = true;
  int n_levels = 0;                 // coarse levels; lv[0] is the first coarse level
  std::vector<glgpu_ctx *> lv;
  struct Transfer
  {
    int32_t *p_ptr = nullptr, *p_idx = nullptr, *r_ptr = nullptr, *r_idx = nullptr;
    void *p_w = nullptr, *r_w = nullptr; // T weights
    TransferSlots p_slots, r_slots;       // the same entries in fixed slots per row (when they fit)
    // Galerkin terms of every coarse block: [g_toff[cb], g_toff[cb+1]) of (fine block, weight)
    int64_t *g_toff = nullptr;
    int32_t *g_row = nullptr, *g_blk = nullptr;
    int32_t *g_up = nullptr, *g_lo = nullptr; // blocks on / above the diagonal; (block, mirror) pairs below
    int64_t n_up = 0, n_lo = 0;
    void *g_w = nullptr;
    std::vector<int32_t> h_ptr, h_idx;   // host copy of P
    std::vector<double> h_w;
  };
  std::vector<Transfer> tr;          // tr[l]: level l (fine side) <-> level l+1
  int64_t *d_dense_off = nullptr;
  float *d_inv = nullptr;
  int *d_sing = nullptr;
  int max_nd = 0;
  void *Zb = nullptr;                // flexible GMRES: preconditioned basis [m][N]
  // the small coarse levels fused into one cooperative launch per V-cycle (level index
  // small_ls .. n_levels; 0: not fused): device descriptors, cycle constants, barrier state
  int small_ls = 0, small_grid = 0;
  void *small_levels = nullptr;
  std::vector<unsigned char> small_cycle; // SmallCycle<T>, passed by value at launch
  unsigned int *small_bar = nullptr;
  int *small_err = nullptr;
  // the V-cycle's tail as one cluster launch per instance (first tail level tail_ls, its
  // parent tail_ls - 1; 0: separate launches): device descriptors, cycle constants, CTAs per
  // cluster
  int tail_ls = 0, tail_cs = 0;
  void *tail_levels = nullptr;
  std::vector<unsigned char> tail_cycle; // TailCycle<T>, passed by value at launch
  void *sinv = nullptr;              // l1 block-Jacobi smoother of the finest level
  bool sinv_half = false;            // ... stored in FP16 (mixed mode, matrix-free operator)
  std::vector<uint8_t> r_ok;         // per instance: R, r_cell, e_cell were evaluated at x
  // per instance, the last glgpu_run step's |R|: the line search's value and the FP64 value
  // that took the stop test (equal in FP64 mode and in steps that did not pass the test)
  std::vector<double> stop_ls, stop_fp64;
  bool mf = false;                   // the Krylov operator is applied matrix-free at the state (FP32, 3D)
  float *ycell = nullptr;            // matrix-free scratch [Nc][8][18]
  float *x32 = nullptr;              // FP32 copy of the state the matrix-free operator linearises at
  bool dinv_ready = false;           // block-Jacobi inverses of the current Jacobian
  bool prec_built = false;           // a multigrid hierarchy exists for some earlier Jacobian
  bool bsr_stale = false;            // the block matrix lags the Hessians (matrix-free steps)
  double last_step_rel = 1e300;      // max over instances of |a delta| / |x| of the last step
  // the V-cycle as a CUDA graph (captured on first use; every pointer it touches is fixed)
  cudaGraphExec_t vc_exec = nullptr;
  void *mg_in = nullptr, *mg_out = nullptr;
  int64_t vc_nodes = 0;
  bool vc_failed = false;
  int64_t mg_fallbacks = 0;          // solves handed from multigrid to block-Jacobi
  // instances whose multigrid solve stalled twice stop where they are instead of finishing
  // with block-Jacobi in this context (mg_handoff); the caller finishes them elsewhere
  bool mg_handoff = false;
  bool reorth = false;               // Gram-Schmidt with one reorthogonalization (default: one projection)
  std::vector<uint8_t> handed;       // per instance, set during the last glgpu_run
};

namespace
{
#define CK(call)                                                                                                     \
  do                                                                                                                 \
    {                                                                                                                \
      cudaError_t e_ = (call);                                                                                       \
      if (e_ != cudaSuccess)                                                                                         \
        return set_error(GLGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                       \
    }                                                                                                                \
  while (0)

#define CKS(call)                                                                                                    \
  do                                                                                                                 \
    {                                                                                                                \
      glgpu_status s_ = (call);                                                                                      \
      if (s_ != GLGPU_OK) return s_;                                                                                 \
    }                                                                                                                \
  while (0)

cudaEvent_t get_event(glgpu_ctx *c)
{
  if (!c->ev_pool.empty())
    {
      cudaEvent_t e = c->ev_pool.back();
      c->ev_pool.pop_back();
      return e;
    }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// harvest finished event pairs into the accumulators (synchronizes on them)
void harvest(glgpu_ctx *c)
{
  for (auto &r : c->kev)
    {
      float ms = 0.f;
      cudaEventSynchronize(r.b);
      if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) c->kms[r.kind] += ms;
      c->ev_pool.push_back(r.a);
      c->ev_pool.push_back(r.b);
    }
  c->kev.clear();
  for (auto &r : c->pev)
    {
      float ms = 0.f;
      cudaEventSynchronize(r.b);
      if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) c->phase_ms[r.kind] += ms;
      c->ev_pool.push_back(r.a);
      c->ev_pool.push_back(r.b);
    }
  c->pev.clear();
}

// launch wrapper: counts launches, optional per-kind event timing
template <typename F> glgpu_status launch(glgpu_ctx *c, int kind, int nk, F &&f)
{
  cudaEvent_t a = nullptr, b = nullptr;
  const bool timed = (c->ktiming >> kind) & 1;
  if (timed)
    {
      a = get_event(c);
      b = get_event(c);
      cudaEventRecord(a, c->st);
    }
  cudaError_t e = f();
  if (e != cudaSuccess) return set_error(GLGPU_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  c->launches += nk;
  c->klaunch[kind] += nk;
  if (timed)
    {
      cudaEventRecord(b, c->st);
      c->kev.push_back({kind, a, b});
      if (c->kev.size() > 4096) harvest(c);
    }
  return GLGPU_OK;
}

struct PhaseScope
{
  glgpu_ctx *c;
  int ph;
  cudaEvent_t a, b;
  PhaseScope(glgpu_ctx *c_, int ph_) : c(c_), ph(ph_)
  {
    a = get_event(c);
    b = get_event(c);
    cudaEventRecord(a, c->st);
  }
  ~PhaseScope()
  {
    cudaEventRecord(b, c->st);
    c->pev.push_back({ph, a, b});
    if (c->pev.size() > 4096) harvest(c);
  }
};

template <typename T> glgpu_status dalloc(glgpu_ctx *c, T **p, size_t n)
{
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T));
  if (e != cudaSuccess)
    return set_error(GLGPU_ERR_NOMEM, "cudaMalloc of " + std::to_string(n * sizeof(T)) + " bytes: " +
                                          cudaGetErrorString(e));
  c->allocs.push_back(*p);
  c->dev_bytes += n * sizeof(T);
  return GLGPU_OK;
}

template <typename T, typename A> glgpu_status dupload(glgpu_ctx *c, T **p, const std::vector<T, A> &v)
{
  CKS(dalloc(c, p, v.size()));
  if (!v.empty()) CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return GLGPU_OK;
}

size_t tsz(const glgpu_ctx *c) { return c->mixed ? sizeof(float) : sizeof(double); }

void *tptr(const glgpu_ctx *c, void *base, int64_t off) { return static_cast<char *>(base) + off * tsz(c); }

glgpu_status sync(glgpu_ctx *c)
{
  cudaError_t e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return set_error(GLGPU_ERR_CUDA, std::string("stream sync: ") + cudaGetErrorString(e));
  return GLGPU_OK;
}

// per-instance 2-norms of a double vector into d_norm and h_norm (synchronizes)
glgpu_status norms_d(glgpu_ctx *c, const double *v, const uint8_t *act, std::vector<double> &out)
{
  CKS(launch(c, KK_VEC, 1,
             [&] { return launch_seg_mdot(c->dm, false, v, 0, 1, v, c->partial, act, c->st); }));
  CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_finalize(c->dm, c->partial, 1, c->d_norm, 1, 1, c->st); }));
  CK(cudaMemcpyAsync(c->h_norm, c->d_norm, sizeof(double) * c->n_inst, cudaMemcpyDeviceToHost, c->st));
  CKS(sync(c));
  out.assign(c->h_norm, c->h_norm + c->n_inst);
  return GLGPU_OK;
}

glgpu_status upload_act(glgpu_ctx *c, uint8_t *dst, const std::vector<uint8_t> &a)
{
  std::memcpy(c->h_act, a.data(), a.size());
  CK(cudaMemcpyAsync(dst, c->h_act, a.size(), cudaMemcpyHostToDevice, c->st));
  CKS(sync(c)); // h_act is reused; keep the copy ordered with the next host write
  return GLGPU_OK;
}

glgpu_status upload_d(glgpu_ctx *c, double *dst, const std::vector<double> &a)
{
  std::memcpy(c->h_res, a.data(), a.size() * sizeof(double));
  CK(cudaMemcpyAsync(dst, c->h_res, a.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
  CKS(sync(c));
  return GLGPU_OK;
}

// Robin face terms into r_cell (and e_cell) at state v, after the cell kernel
glgpu_status robin_res(glgpu_ctx *c, const double *v, double *ec, const uint8_t *act)
{
  if (c->dm.n_robin == 0) return GLGPU_OK;
  return launch(c, KK_RES, 1, [&] { return launch_robin_res(c->dm, v, c->r_cell, ec, act, c->st); });
}

// kernels of one matrix-free operator application: cell, (Robin faces,) gather
int mf_launches(const glgpu_ctx *c) { return 2 + (c->dm.n_robin > 0 ? 1 : 0); }

// R at v (x or xt) for the instances in act, and the cell free energies when `energy` (the
// line search needs only |R|).  Mixed contexts evaluate it in double-float arithmetic unless
// `fp64`: the FP64 kernel certifies the stop test and gives the free energy.
glgpu_status residual_at(glgpu_ctx *c, const double *v, const uint8_t *act, bool energy = false, bool fp64 = false)
{
  double *ec = energy ? c->e_cell : nullptr;
  const bool df = c->mixed && !fp64;
  CKS(launch(c, KK_RES, 1, [&] { return launch_cell(c->dm, df, v, nullptr, c->r_cell, ec, act, c->st); }));
  CKS(robin_res(c, v, ec, act));
  CKS(launch(c, KK_RES, 1, [&] { return launch_res_gather(c->dm, c->r_cell, c->R, act, c->st); }));
  return GLGPU_OK;
}

// ---------------------------------------------------------------------------------
// preconditioner
// ---------------------------------------------------------------------------------
glgpu_status bj(glgpu_ctx *c, const void *in, void *out, const uint8_t *act, const void *inv = nullptr)
{
  const void *d = inv ? inv : c->dinv;
  return launch(c, KK_PREC, 1, [&] { return launch_bj_apply(c->dm, c->mixed, d, in, out, act, c->st); });
}

glgpu_status spmv(glgpu_ctx *c, const void *in, void *out, const uint8_t *act)
{
  if (c->mf)
    return launch(c, KK_SPMV, mf_launches(c), [&] {
      return launch_mf(c->dm, c->x32, static_cast<const float *>(in), c->ycell,
                       static_cast<float *>(out), nullptr, nullptr, 0.f, 0, act, c->st, c->prm[0].mf_cells);
    });
  return launch(c, KK_SPMV, 1, [&] { return launch_spmv(c->dm, c->mixed, c->vals, in, out, act, c->st); });
}

glgpu_status axpby(glgpu_ctx *c, const void *x, void *y, const void *z, const Axpby &k, const uint8_t *act,
                   bool x32, bool y32, bool z32)
{
  return launch(c, KK_VEC, 1, [&] { return launch_seg_axpby(c->dm, x32, x, y32, y, z32, z, k, act, c->st); });
}

Axpby coefs(double a, double b, double cc = 0.0)
{
  Axpby k{};
  k.a0 = a;
  k.b0 = b;
  k.c0 = cc;
  return k;
}

// Chebyshev coefficients per instance: d_cheb[k][0..1] = theta, delta
glgpu_status cheb_setup(glgpu_ctx *c)
{
  const bool m = c->mixed;
  const int n_inst = c->n_inst;
  // power iteration on D^-1 J, 12 steps, deterministic start vector of ones (Dirichlet zeros kept)
  CKS(axpby(c, nullptr, c->C1, nullptr, coefs(0.0, 0.0), nullptr, m, m, m));
  // C1 = 1 everywhere: use y = a*x + b*y with x = NULL is zero; set via z trick: use Tmp
  {
    std::vector<double> ones(c->N, 1.0);
    double *tmpd = c->xt; // scratch double vector
    CK(cudaMemcpyAsync(tmpd, ones.data(), sizeof(double) * c->N, cudaMemcpyHostToDevice, c->st));
    CK(launch_distribute(c->dm, tmpd, c->st));
    c->launches += 2;
    CKS(axpby(c, tmpd, c->C1, nullptr, coefs(1.0, 0.0), nullptr, false, m, m));
    CKS(sync(c));
  }
  std::vector<double> lam(n_inst, 1.0);
  for (int it = 0; it < 12; ++it)
    {
      CKS(spmv(c, c->C1, c->C2, nullptr));
      CKS(bj(c, c->C2, c->C3, nullptr));
      // norms of C3 and C1
      CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_mdot(c->dm, m, c->C3, 0, 1, c->C3, c->partial, nullptr, c->st); }));
      CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_finalize(c->dm, c->partial, 1, c->d_norm, 1, 1, c->st); }));
      CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_mdot(c->dm, m, c->C1, 0, 1, c->C1, c->partial, nullptr, c->st); }));
      CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_finalize(c->dm, c->partial, 1, c->d_tmp, 1, 1, c->st); }));
      CK(cudaMemcpyAsync(c->h_norm, c->d_norm, sizeof(double) * n_inst, cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(c->h_res, c->d_tmp, sizeof(double) * n_inst, cudaMemcpyDeviceToHost, c->st));
      CKS(sync(c));
      for (int k = 0; k < n_inst; ++k) lam[k] = (c->h_res[k] > 0) ? c->h_norm[k] / c->h_res[k] : 1.0;
      // C1 = C3 / |C3|
      CKS(launch(c, KK_VEC, 1, [&] { return launch_inv(c->d_norm, c->d_tmp, n_inst, c->st); }));
      Axpby k{};
      k.a = c->d_tmp;
      k.sa = 1;
      k.b0 = 0.0;
      CKS(axpby(c, c->C3, c->C1, nullptr, k, nullptr, m, m, m));
    }
  c->lam_max.resize(n_inst);
  std::vector<double> tc(2 * n_inst);
  for (int k = 0; k < n_inst; ++k)
    {
      const double lmax = 1.1 * lam[k];
      const double lmin = lmax / 30.0;
      c->lam_max[k] = lmax;
      tc[2 * k] = 0.5 * (lmax + lmin);
      tc[2 * k + 1] = 0.5 * (lmax - lmin);
    }
  std::memcpy(c->h_res, tc.data(), sizeof(double) * 2 * n_inst);
  CK(cudaMemcpyAsync(c->d_cheb, c->h_res, sizeof(double) * 2 * n_inst, cudaMemcpyHostToDevice, c->st));
  CKS(sync(c));
  return GLGPU_OK;
}

// z = M^-1 v
glgpu_status precond(glgpu_ctx *c, const void *v, void *z, const uint8_t *act)
{
  const bool m = c->mixed;
  const int pc = c->prm[0].precond;
  if (pc == GLGPU_PC_NONE) return axpby(c, v, z, nullptr, coefs(1.0, 0.0), act, m, m, m);
  // multigrid contexts fall back to block-Jacobi (refined meshes, stalled cycles)
  if (pc == GLGPU_PC_BLOCK_JACOBI || pc == GLGPU_PC_MULTIGRID) return bj(c, v, z, act);
  // Chebyshev semi-iteration for J z = v preconditioned by D^-1, started at z = 0.
  // Step scalars per instance live at d_cheb + 2 n_inst as [deg][n_inst][2]:
  // step 0 uses (0, 1/theta), step i >= 1 uses (rho_i rho_{i-1}, 2 rho_i / delta).
  const int deg = std::max(1, c->prm[0].cheb_degree);
  const double *sc = c->d_cheb + 2 * c->n_inst;
  CKS(axpby(c, v, c->C1, nullptr, coefs(1.0, 0.0), act, m, m, m)); // r = v
  CKS(bj(c, c->C1, c->C2, act));                                     // d = D^-1 r
  {
    Axpby k{};
    k.a = sc + 1;
    k.sa = 2;
    CKS(axpby(c, c->C2, c->C2, nullptr, k, act, m, m, m)); // d = d / theta
  }
  CKS(axpby(c, c->C2, z, nullptr, coefs(1.0, 0.0), act, m, m, m)); // z = d
  for (int i = 1; i < deg; ++i)
    {
      CKS(spmv(c, c->C2, c->C3, act));                                       // C3 = J d
      CKS(axpby(c, c->C3, c->C1, nullptr, coefs(-1.0, 1.0), act, m, m, m));  // r -= J d
      CKS(bj(c, c->C1, c->C3, act));                                         // C3 = D^-1 r
      Axpby k{};
      k.b = sc + static_cast<int64_t>(i) * 2 * c->n_inst;
      k.sb = 2;
      k.a = sc + static_cast<int64_t>(i) * 2 * c->n_inst + 1;
      k.sa = 2;
      CKS(axpby(c, c->C3, c->C2, nullptr, k, act, m, m, m));                 // d = c_d d + c_r D^-1 r
      CKS(axpby(c, c->C2, z, nullptr, coefs(1.0, 1.0), act, m, m, m));       // z += d
    }
  return GLGPU_OK;
}

glgpu_status cheb_coeffs(glgpu_ctx *c)
{
  const int deg = std::max(1, c->prm[0].cheb_degree);
  const int n = c->n_inst;
  std::vector<double> tcv(2 * n);
  CK(cudaMemcpy(tcv.data(), c->d_cheb, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
  std::vector<double> sc(static_cast<size_t>(deg) * 2 * n, 0.0);
  for (int k = 0; k < n; ++k)
    {
      const double theta = tcv[2 * k], delta = tcv[2 * k + 1];
      const double sigma = theta / delta;
      double rho_old = 1.0 / sigma;
      sc[2 * k + 0] = 0.0;
      sc[2 * k + 1] = 1.0 / theta;
      for (int i = 1; i < deg; ++i)
        {
          const double rho = 1.0 / (2.0 * sigma - rho_old);
          sc[(static_cast<size_t>(i) * n + k) * 2 + 0] = rho * rho_old;
          sc[(static_cast<size_t>(i) * n + k) * 2 + 1] = 2.0 * rho / delta;
          rho_old = rho;
        }
    }
  CK(cudaMemcpy(c->d_cheb + 2 * n, sc.data(), sizeof(double) * sc.size(), cudaMemcpyHostToDevice));
  return GLGPU_OK;
}

glgpu_status mg_assemble(glgpu_ctx *c, const uint8_t *act);

glgpu_status bj_setup(glgpu_ctx *c)
{
  if (c->dinv_ready) return GLGPU_OK;
  CKS(launch(c, KK_PREC, 1, [&] { return launch_bj_setup(c->dm, c->mixed, c->vals, c->dinv, c->st); }));
  c->dinv_ready = true;
  return GLGPU_OK;
}

// Preconditioner setup for the current Jacobian (the reference builds its AMG inside
// solve, solve.cc:141-152): the multigrid hierarchy, or the block-Jacobi inverses
// (multigrid computes those only when a solve falls back to them).
glgpu_status prec_setup(glgpu_ctx *c, const uint8_t *act)
{
  if (c->prec_ready) return GLGPU_OK;
  const int pc = c->prm[0].precond;
  if (pc == GLGPU_PC_MULTIGRID && c->n_levels > 0)
    {
      CKS(mg_assemble(c, act));
      c->prec_built = true;
    }
  else if (pc >= GLGPU_PC_BLOCK_JACOBI)
    CKS(bj_setup(c));
  if (pc == GLGPU_PC_CHEBYSHEV)
    {
      CKS(cheb_setup(c));
      CKS(cheb_coeffs(c));
    }
  c->prec_ready = true;
  return GLGPU_OK;
}

// pre_done: z already holds the first sweep from zero (omega D^-1 r, fused with the restriction)
glgpu_status vcycle(glgpu_ctx *c, int l, const void *r, void *z, const uint8_t *act, bool pre_done = false);

// z = V-cycle(r) for the flexible GMRES basis, masked by the GMRES activity flags.  The
// cycle's ~9 launches per level are captured once into a CUDA graph over fixed input and
// output buffers and replayed; if capture is unavailable the cycle runs launch by launch.
glgpu_status vcycle_run(glgpu_ctx *c, const void *r, void *z)
{
  const size_t bytes = tsz(c) * static_cast<size_t>(c->N);
  if (!c->vc_exec && !c->vc_failed)
    {
      std::vector<glgpu_ctx *> all(1, c);
      all.insert(all.end(), c->lv.begin(), c->lv.end());
      std::vector<int64_t> l0, k0;
      std::vector<int> t0;
      for (glgpu_ctx *x : all)
        {
          l0.push_back(x->launches);
          for (int k = 0; k < KK_N; ++k) k0.push_back(x->klaunch[k]);
          t0.push_back(x->ktiming);
          x->ktiming = 0;
        }
      cudaGraph_t g = nullptr;
      glgpu_status st = GLGPU_OK;
      if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        st = GLGPU_ERR_CUDA;
      else
        {
          st = vcycle(c, 0, c->mg_in, c->mg_out, c->g.active);
          if (cudaStreamEndCapture(c->st, &g) != cudaSuccess) st = GLGPU_ERR_CUDA;
        }
      if (st == GLGPU_OK && g && cudaGraphInstantiate(&c->vc_exec, g, 0) != cudaSuccess) c->vc_exec = nullptr;
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      int64_t nodes = 0;
      for (size_t i = 0; i < all.size(); ++i)
        {
          nodes += all[i]->launches - l0[i];
          all[i]->launches = l0[i];
          for (int k = 0; k < KK_N; ++k) all[i]->klaunch[k] = k0[i * KK_N + k];
          all[i]->ktiming = t0[i];
        }
      c->vc_nodes = nodes;
      if (!c->vc_exec) c->vc_failed = true;
    }
  if (!c->vc_exec) return vcycle(c, 0, r, z, c->g.active);
  CK(cudaMemcpyAsync(c->mg_in, r, bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaGraphLaunch(c->vc_exec, c->st));
  CK(cudaMemcpyAsync(z, c->mg_out, bytes, cudaMemcpyDeviceToDevice, c->st));
  c->launches += c->vc_nodes;
  return GLGPU_OK;
}

// ---------------------------------------------------------------------------------
// GMRES(m), right preconditioned, classical Gram-Schmidt with one reorthogonalization
// ---------------------------------------------------------------------------------
constexpr double kMgStall = 0.5; // least reduction of the true residual per multigrid cycle

glgpu_status gmres(glgpu_ctx *c, double tol, const std::vector<uint8_t> &on, std::vector<int> &its_out,
                   bool &all_conv)
{
  const bool m32 = c->mixed;
  const int n = c->n_inst, mr = c->restart;
  const int64_t N = c->N;
  const int maxit = std::max(1, c->prm[0].gmres_max_iter);
  std::vector<double> tol_abs(n);
  for (int k = 0; k < n; ++k) tol_abs[k] = tol * c->rhs_norm[k];
  CKS(upload_d(c, c->g.tol, tol_abs));
  CKS(upload_act(c, c->d_act2, on));
  // b in Krylov precision, X = 0
  CKS(axpby(c, c->rhs, c->Bv, nullptr, coefs(1.0, 0.0), nullptr, false, m32, m32));
  CKS(axpby(c, nullptr, c->X, nullptr, coefs(0.0, 0.0), nullptr, m32, m32, m32));
  std::vector<int> total(n, 0);
  std::vector<uint8_t> solve_on(on);
  std::vector<uint8_t> deferred(static_cast<size_t>(n), 0); // set aside (multigrid retry, then block-Jacobi)
  bool mg_retried = false;
  all_conv = false;
  // multigrid runs flexible GMRES; an instance whose restart cycle does not at least halve its
  // true residual is set aside, retried with a fresh multigrid pass once the others are done,
  // and finished with block-Jacobi GMRES if it stalls again
  bool use_mg = c->n_levels > 0;
  std::vector<double> prev_res(c->rhs_norm);
  for (int cycle = 0;; ++cycle)
    {
      // V0 = b - J X
      if (cycle == 0)
        CKS(axpby(c, c->Bv, c->V, nullptr, coefs(1.0, 0.0), c->d_act2, m32, m32, m32));
      else
        {
          CKS(spmv(c, c->X, c->Tmp, c->d_act2));
          CKS(axpby(c, c->Bv, c->V, c->Tmp, coefs(1.0, 0.0, -1.0), c->d_act2, m32, m32, m32));
        }
      CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_mdot(c->dm, m32, c->V, 0, 1, c->V, c->partial, c->d_act2, c->st); }));
      CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_finalize(c->dm, c->partial, 1, c->g.beta, 1, 1, c->st); }));
      CKS(launch(c, KK_VEC, 1, [&] { return launch_gmres_start(c->g, n, c->d_act2, c->st); }));
      {
        Axpby k{};
        k.a = c->g.inv_scale;
        k.sa = 1;
        CKS(axpby(c, c->V, c->V, nullptr, k, c->g.active, m32, m32, m32));
      }
      CK(cudaMemcpyAsync(c->h_act, c->g.active, n, cudaMemcpyDeviceToHost, c->st));
      CKS(sync(c));
      bool any = false;
      for (int k = 0; k < n; ++k) any |= c->h_act[k] != 0;
      if (!any)
        {
          all_conv = true;
          break;
        }
      int jdone = 0;
      for (int j = 0; j < mr; ++j)
        {
          void *Vj = tptr(c, c->V, static_cast<int64_t>(j) * N);
          void *Vj1 = tptr(c, c->V, static_cast<int64_t>(j + 1) * N);
          // fused path: the normalisation of V_j is folded into the block-Jacobi pass and
          // the Gram-Schmidt finalisation and Givens update run inside the reductions.
          // Multigrid (flexible GMRES): Z_j = V-cycle(V_j) is kept for the solution update.
          const bool mg = use_mg;
          const bool fused_bj = !mg && c->B == 18 &&
                                (c->prm[0].precond == GLGPU_PC_BLOCK_JACOBI || c->prm[0].precond == GLGPU_PC_MULTIGRID);
          const bool fused = fused_bj || mg;
          void *Zj = mg ? tptr(c, c->Zb, static_cast<int64_t>(j) * N) : c->Z;
          if (fused_bj)
            {
              const double *sc = (j == 0) ? nullptr : c->g.inv_scale;
              CKS(launch(c, KK_PREC, 1, [&] {
                return launch_bj_apply_scale(c->dm, m32, c->dinv, Vj, c->Z, sc, c->g.active, c->st);
              }));
            }
          else if (mg)
            CKS(vcycle_run(c, Vj, Zj));
          else
            CKS(precond(c, Vj, c->Z, c->g.active));
          CKS(spmv(c, Zj, Vj1, c->g.active));
          if (fused)
            {
              CKS(launch(c, KK_VEC, 1, [&] {
                return launch_arnoldi_dot(c->dm, m32, c->V, N, j + 1, Vj1, c->partial, c->g.hcol, mr + 2, c->d_cnt,
                                          c->g.active, c->st);
              }));
              if (c->reorth)
                {
                  CKS(launch(c, KK_VEC, 1, [&] {
                    return launch_arnoldi_update(c->dm, m32, c->V, N, j + 1, Vj1, 1, j, c->partial, c->g, c->d_cnt,
                                                 c->st);
                  }));
                  CKS(launch(c, KK_VEC, 1, [&] {
                    return launch_arnoldi_update(c->dm, m32, c->V, N, j + 1, Vj1, 2, j, c->partial, c->g, c->d_cnt,
                                                 c->st);
                  }));
                }
              else
                CKS(launch(c, KK_VEC, 1, [&] {
                  return launch_arnoldi_update(c->dm, m32, c->V, N, j + 1, Vj1, 3, j, c->partial, c->g, c->d_cnt, c->st);
                }));
              if (mg)
                {
                  Axpby k{};
                  k.a = c->g.inv_scale;
                  k.sa = 1;
                  CKS(axpby(c, Vj1, Vj1, nullptr, k, c->g.active, m32, m32, m32));
                }
            }
          else
            {
              // classical Gram-Schmidt with one reorthogonalization; the second projection
              // and the norm come out of the update passes (3 reads of the basis, not 4)
              CKS(launch(c, KK_VEC, 1, [&] {
                return launch_seg_mdot(c->dm, m32, c->V, N, j + 1, Vj1, c->partial, c->g.active, c->st);
              }));
              CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_finalize(c->dm, c->partial, j + 1, c->g.hcol, mr + 2, 0, c->st); }));
              CKS(launch(c, KK_VEC, 1, [&] {
                return launch_seg_update(c->dm, m32, c->V, N, j + 1, c->g.hcol, mr + 2, Vj1, j + 1, c->partial, nullptr,
                                         c->g.active, c->st);
              }));
              CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_finalize(c->dm, c->partial, j + 1, c->g.hcol2, mr + 2, 0, c->st); }));
              CKS(launch(c, KK_VEC, 1, [&] {
                return launch_seg_update(c->dm, m32, c->V, N, j + 1, c->g.hcol2, mr + 2, Vj1, 0, nullptr, c->partial_n,
                                         c->g.active, c->st);
              }));
              CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_finalize(c->dm, c->partial_n, 1, c->g.hcol + j + 1, mr + 2, 1, c->st); }));
              CKS(launch(c, KK_VEC, 1, [&] { return launch_gmres_column(c->g, n, j, c->st); }));
              Axpby k{};
              k.a = c->g.inv_scale;
              k.sa = 1;
              CKS(axpby(c, Vj1, Vj1, nullptr, k, c->g.active, m32, m32, m32));
            }
          jdone = j + 1;
          // step j's flags are copied out and checked only after step j+1 is enqueued,
          // so the host round trip overlaps device work; instances that stopped are
          // masked on the device, which makes a speculative step a no-op for them
          uint8_t *slot = c->h_act_pipe + (j & 1) * n;
          CK(cudaMemcpyAsync(slot, c->g.active, n, cudaMemcpyDeviceToHost, c->st));
          CK(cudaEventRecord(c->ev_pipe[j & 1], c->st));
          if (j >= 1)
            {
              CK(cudaEventSynchronize(c->ev_pipe[(j - 1) & 1]));
              const uint8_t *prev = c->h_act_pipe + ((j - 1) & 1) * n;
              bool anyj = false;
              for (int k = 0; k < n; ++k) anyj |= prev[k] != 0;
              if (!anyj) break;
            }
        }
      // X += M^-1 (V y), or X += Z y for flexible GMRES (y is stored negated)
      CKS(launch(c, KK_VEC, 1, [&] { return launch_gmres_solve_y(c->g, n, c->st); }));
      if (use_mg)
        CKS(launch(c, KK_VEC, 1, [&] {
          return launch_seg_maxpy(c->dm, m32, c->Zb, N, jdone, c->g.y, mr, c->X, c->d_act2, c->st);
        }));
      else
        {
          CKS(axpby(c, nullptr, c->Tmp, nullptr, coefs(0.0, 0.0), c->d_act2, m32, m32, m32));
          CKS(launch(c, KK_VEC, 1, [&] {
            return launch_seg_maxpy(c->dm, m32, c->V, N, jdone, c->g.y, mr, c->Tmp, c->d_act2, c->st);
          }));
          CKS(precond(c, c->Tmp, c->Z, c->d_act2));
          CKS(axpby(c, c->Z, c->X, nullptr, coefs(1.0, 1.0), c->d_act2, m32, m32, m32));
        }
      CK(cudaMemcpyAsync(c->h_its, c->g.its, sizeof(int) * n, cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(c->h_norm, c->g.res_est, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st));
      if (use_mg)
        {
          // flexible GMRES can stop on a breakdown of the preconditioned basis with a small
          // estimate: measure the cycle by the true residual |b - J X| instead
          CKS(spmv(c, c->X, c->Tmp, c->d_act2));
          CKS(axpby(c, c->Bv, c->Tmp, nullptr, coefs(1.0, -1.0), c->d_act2, m32, m32, m32));
          CKS(launch(c, KK_VEC, 1, [&] {
            return launch_seg_mdot(c->dm, m32, c->Tmp, 0, 1, c->Tmp, c->partial, c->d_act2, c->st);
          }));
          CKS(launch(c, KK_VEC, 1, [&] { return launch_seg_finalize(c->dm, c->partial, 1, c->d_tmp, 1, 1, c->st); }));
          CK(cudaMemcpyAsync(c->h_norm, c->d_tmp, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st));
        }
      CKS(sync(c));
      if (use_mg)
        {
          std::vector<uint8_t> bad(n, 0);
          bool any_bad = false;
          for (int k = 0; k < n; ++k)
            {
              if (!solve_on[k] || c->h_norm[k] <= tol_abs[k]) continue;
              if (!std::isfinite(c->h_norm[k]) || c->h_norm[k] > prev_res[k])
                {
                  bad[k] = 1;
                  any_bad = true;
                }
              else if (c->h_norm[k] > kMgStall * prev_res[k])
                deferred[k] = 1;
            }
          if (any_bad)
            {
              // the cycle made things worse: restart these instances from X = 0
              CKS(upload_act(c, c->d_act2, bad));
              CKS(axpby(c, nullptr, c->X, nullptr, coefs(0.0, 0.0), c->d_act2, m32, m32, m32));
              for (int k = 0; k < n; ++k)
                if (bad[k]) c->h_norm[k] = c->rhs_norm[k];
            }
          for (int k = 0; k < n; ++k)
            if (solve_on[k]) prev_res[k] = c->h_norm[k];
          // an instance whose cycle diverged or stalled leaves the multigrid solve; it is
          // finished with block-Jacobi GMRES once the other instances have converged, so one
          // hard instance does not slow the rest of its batch
          for (int k = 0; k < n; ++k)
            if (bad[k]) deferred[k] = 1;
        }
      bool more = false;
      for (int k = 0; k < n; ++k)
        {
          if (!solve_on[k]) continue;
          total[k] += c->h_its[k];
          const bool conv = c->h_norm[k] <= tol_abs[k];
          if (conv || total[k] >= maxit || !std::isfinite(c->h_norm[k]))
            {
              solve_on[k] = 0;
              deferred[k] = 0;
            }
          else if (deferred[k])
            solve_on[k] = 0; // set aside for the block-Jacobi pass
          else
            more = true;
        }
      if (!more && use_mg)
        {
          bool any_def = false;
          for (int k = 0; k < n; ++k) any_def |= deferred[k] != 0;
          if (any_def && !mg_retried)
            {
              // first the set-aside instances get one fresh multigrid pass from their current X
              // (a stall of flexible GMRES can be a poor Krylov space rather than a failing
              // V-cycle); those that stall again finish with block-Jacobi
              mg_retried = true;
              for (int k = 0; k < n; ++k)
                if (deferred[k]) prev_res[k] = c->h_norm[k];
              solve_on = deferred;
              std::fill(deferred.begin(), deferred.end(), 0);
              more = true;
            }
          else if (any_def && c->mg_handoff)
            {
              // handed off: these instances leave the solve with the X they reached; the
              // Newton loop stops them without an update
              for (int k = 0; k < n; ++k)
                if (deferred[k]) c->handed[k] = 1;
              std::fill(deferred.begin(), deferred.end(), 0);
            }
          else if (any_def)
            {
              // the set-aside instances continue from their current X with block-Jacobi GMRES
              use_mg = false;
              c->mg_fallbacks++;
              CKS(bj_setup(c));
              solve_on = deferred;
              std::fill(deferred.begin(), deferred.end(), 0);
              more = true;
            }
        }
      if (!more)
        {
          // converged unless an instance ran out of iterations: verify with the true residual
          all_conv = true;
          for (int k = 0; k < n; ++k)
            if (on[k] && (total[k] >= maxit && c->h_norm[k] > tol_abs[k])) all_conv = false;
          break;
        }
      CKS(upload_act(c, c->d_act2, solve_on));
    }
  // delta = X (double), distributed through the constraints
  CKS(axpby(c, c->X, c->delta, nullptr, coefs(1.0, 0.0), nullptr, m32, false, false));
  CK(launch_distribute(c->dm, c->delta, c->st));
  c->launches += 2;
  its_out = total;
  return GLGPU_OK;
}

// ---------------------------------------------------------------------------------
// geometric multigrid
// ---------------------------------------------------------------------------------
template <typename T> glgpu_status upload_w(glgpu_ctx *c, void **dst, const std::vector<double> &w)
{
  std::vector<T> tw(w.begin(), w.end());
  T *p = nullptr;
  CKS(dupload(c, &p, tw));
  *dst = p;
  return GLGPU_OK;
}

// after the fine assembly: the l1 block-Jacobi smoother of the finest level, coarse
// Jacobians P^T J P level by level with their l1 smoothers, and the dense inverse of
// the coarsest level
glgpu_status mg_assemble(glgpu_ctx *c, const uint8_t *act)
{
  CKS(launch(c, KK_PREC, 1, [&] {
    return c->sinv_half ? launch_bj_setup_half(c->dm, c->vals, static_cast<__half *>(c->sinv), c->st)
                        : launch_bj_setup(c->dm, c->mixed, c->vals, c->sinv, c->st, true);
  }));
  for (int l = 0; l < c->n_levels; ++l)
    {
      glgpu_ctx *F = (l == 0) ? c : c->lv[l - 1];
      glgpu_ctx *L = c->lv[l];
      const glgpu_ctx::Transfer &t = c->tr[l];
      CKS(launch(c, KK_PREC, 1, [&] {
        return launch_galerkin(c->mixed, t.n_up, t.g_up, t.n_lo, t.g_lo, t.g_row, L->dm.cols, L->dm.mask, L->dm.hptr,
                               L->vals, t.g_toff, t.g_blk, t.g_w, F->vals, L->dm.node_inst, act, c->st,
                               F->dm.half_vals != 0, L->dm.half_vals != 0);
      }));
      CKS(launch(c, KK_PREC, 1, [&] { return launch_bj_setup(L->dm, L->mixed, L->vals, L->dinv, L->st, true); }));
      L->has_J = true;
    }
  glgpu_ctx *Lc = c->lv[c->n_levels - 1];
  CKS(launch(c, KK_PREC, 1, [&] {
    return launch_dense_setup(Lc->dm, c->mixed, Lc->vals, c->d_dense_off, c->max_nd, c->d_inv, c->d_sing,
                              static_cast<float>(c->prm[0].mg_coarse_shift), c->st);
  }));
  return GLGPU_OK;
}

// z = V-cycle(r) on level l (l = 0: this context); r, z in the Krylov precision.
// Per level: smoothing sweeps are fused kernels (y = z + omega D1^-1 (r - J z), D1 the
// l1 block-Jacobi blocks), the residual is the SpMV's residual form, and the coarse
// correction is written next to the smoothed iterate, so the buffers ping-pong instead
// of being copied.
glgpu_status vcycle(glgpu_ctx *c, int l, const void *r, void *z, const uint8_t *act, bool pre_done)
{
  const bool m = c->mixed;
  if (l > 0 && l == c->small_ls && pre_done)
    // this level and every coarser one in one cooperative launch (r, z are this level's
    // Bv and X, which the descriptors hold)
    return launch(c, KK_PREC, 1, [&] {
      return launch_vcycle_small(m, c->small_levels, c->small_cycle.data(), c->small_grid, act, c->st);
    });
  if (l == c->n_levels)
    {
      glgpu_ctx *L = c->lv[l - 1];
      return launch(c, KK_PREC, 1, [&] {
        return launch_dense_apply(L->dm, m, c->max_nd, c->d_dense_off, c->d_inv, r, z, act, c->st);
      });
    }
  glgpu_ctx *L = (l == 0) ? c : c->lv[l - 1];
  const void *sm = (l == 0) ? c->sinv : L->dinv; // l1 block-Jacobi
  void *t = (l == 0) ? c->C2 : L->Tmp;
  void *t2 = (l == 0) ? c->C3 : L->C1;
  const double om = c->prm[0].mg_omega;
  const int pre = std::max(1, c->prm[0].mg_pre), post = std::max(0, c->prm[0].mg_post);
  const bool half_sm = (l == 0) && c->sinv_half;
  auto smooth = [&](const void *zin, void *zout) {
    if (L->mf && zin)
      return launch(L, KK_PREC, mf_launches(L), [&] {
        return launch_mf(L->dm, L->x32, static_cast<const float *>(zin), L->ycell,
                         static_cast<float *>(zout), static_cast<const float *>(r), static_cast<const __half *>(sm),
                         static_cast<float>(om), 2, act, L->st, L->prm[0].mf_cells);
      });
    if (half_sm && !zin)
      return launch(L, KK_PREC, 1, [&] {
        return launch_smooth_zero_half(L->dm, static_cast<const __half *>(sm), static_cast<const float *>(r),
                                       static_cast<float *>(zout), om, act, L->st);
      });
    return launch(L, KK_PREC, 1, [&] { return launch_smooth(L->dm, m, L->vals, sm, r, zin, zout, om, act, L->st); });
  };
  // pre-smoothing from zero, ping-ponging between z and t2; `cur` holds the iterate
  void *cur = z, *oth = t2;
  if (!pre_done) CKS(smooth(nullptr, cur));
  for (int s = 1; s < pre; ++s)
    {
      CKS(smooth(cur, oth));
      std::swap(cur, oth);
    }
  // coarse-grid correction: oth = cur + P e, e = V-cycle(R (r - J cur))
  if (L->mf)
    CKS(launch(L, KK_SPMV, mf_launches(L), [&] {
      return launch_mf(L->dm, L->x32, static_cast<const float *>(cur), L->ycell,
                       static_cast<float *>(t), static_cast<const float *>(r), nullptr, 0.f, 1, act, L->st, L->prm[0].mf_cells);
    }));
  else
    CKS(launch(L, KK_SPMV, 1, [&] { return launch_spmv(L->dm, m, L->vals, cur, t, act, L->st, r); }));
  glgpu_ctx *C = c->lv[l];
  const glgpu_ctx::Transfer &tr = c->tr[l];
  if (c->tail_ls == l + 1)
    // every coarser level in one cluster launch per instance, ending with oth = cur + P e
    CKS(launch(c, KK_PREC, 1, [&] {
      return launch_vcycle_tail(m, c->tail_levels, c->tail_cycle.data(), c->n_inst, c->tail_cs, t, cur, oth, act,
                                c->st);
    }));
  else
    {
      const bool fuse = (l + 1 < c->n_levels) && C->B == 18; // the next level smooths (not the dense solve)
      if (fuse)
        CKS(launch(c, KK_PREC, 1, [&] {
          return launch_restrict_smooth(m, C->nn, tr.r_ptr, tr.r_idx, tr.r_w, t, C->Bv, C->dm.mask, C->dm.node_inst,
                                        act, C->dinv, om, C->X, c->st, tr.r_slots);
        }));
      else
        CKS(launch(c, KK_PREC, 1, [&] {
          return launch_restrict(m, C->nn, C->B, tr.r_ptr, tr.r_idx, tr.r_w, t, C->Bv, C->dm.mask,
                                 C->dm.node_inst, act, c->st, tr.r_slots);
        }));
      CKS(vcycle(c, l + 1, C->Bv, C->X, act, fuse));
      CKS(launch(c, KK_PREC, 1, [&] {
        return launch_prolong(m, L->nn, L->B, tr.p_ptr, tr.p_idx, tr.p_w, C->X, oth, L->dm.mask, L->dm.hptr,
                              L->dm.node_inst, act, c->st, cur, tr.p_slots);
      }));
    }
  std::swap(cur, oth);
  for (int s = 0; s < post; ++s)
    {
      CKS(smooth(cur, oth));
      std::swap(cur, oth);
    }
  if (cur != z) CKS(axpby(L, cur, z, nullptr, coefs(1.0, 0.0), act, m, m, m));
  return GLGPU_OK;
}

// Small coarse levels below which one cooperative launch runs the rest of the V-cycle:
// levels of at most kSmallNodes nodes (all instances together), FP32/FP64 blocks, down
// to the dense coarsest level.
constexpr int64_t kSmallNodes = 20000;

template <typename T> glgpu_status small_setup_t(glgpu_ctx *c, int ls)
{
  const int nl = c->n_levels;
  std::vector<SmallLevel<T>> lev(static_cast<size_t>(nl - ls + 1));
  for (int l = ls; l <= nl; ++l)
    {
      glgpu_ctx *L = c->lv[l - 1];
      SmallLevel<T> &d = lev[static_cast<size_t>(l - ls)];
      d.m = L->dm;
      d.vals = static_cast<const T *>(L->vals);
      d.dinv = static_cast<const T *>(L->dinv);
      d.r = static_cast<T *>(L->Bv);
      d.z = static_cast<T *>(L->X);
      d.t = static_cast<T *>(L->Tmp);
      d.t2 = static_cast<T *>(L->C1);
      if (l < nl)
        {
          const glgpu_ctx::Transfer &t = c->tr[l];
          d.r_ptr = t.r_ptr;
          d.r_idx = t.r_idx;
          d.r_w = static_cast<const T *>(t.r_w);
          d.p_ptr = t.p_ptr;
          d.p_idx = t.p_idx;
          d.p_w = static_cast<const T *>(t.p_w);
        }
    }
  std::vector<unsigned char> bytes(sizeof(SmallLevel<T>) * lev.size());
  std::memcpy(bytes.data(), lev.data(), bytes.size());
  unsigned char *dl = nullptr;
  CKS(dupload(c, &dl, bytes));
  c->small_levels = dl;
  CKS(dalloc(c, &c->small_bar, 2));
  CKS(dalloc(c, &c->small_err, 1));
  CK(cudaMemset(c->small_bar, 0, 2 * sizeof(unsigned int)));
  CK(cudaMemset(c->small_err, 0, sizeof(int)));
  SmallCycle<T> cy{};
  cy.n_small = nl - ls;
  cy.pre = std::max(1, c->prm[0].mg_pre);
  cy.post = std::max(0, c->prm[0].mg_post);
  cy.omega = static_cast<T>(c->prm[0].mg_omega);
  cy.max_nd = c->max_nd;
  cy.dense_off = c->d_dense_off;
  cy.inv = c->d_inv;
  cy.bar = c->small_bar;
  cy.err = c->small_err;
  c->small_cycle.resize(sizeof(cy));
  std::memcpy(c->small_cycle.data(), &cy, sizeof(cy));
  c->small_ls = ls;
  return GLGPU_OK;
}

glgpu_status small_setup(glgpu_ctx *c)
{
  const int nl = c->n_levels;
  if (nl < 2 || c->B != 18 || c->prm[0].mg_small_fuse != 1) return GLGPU_OK;
  int ls = nl;
  while (ls - 1 >= 1)
    {
      const glgpu_ctx *L = c->lv[ls - 2]; // level ls - 1
      if (L->nn > kSmallNodes || L->dm.half_vals || L->B != 18) break;
      --ls;
    }
  ls = std::max(ls, nl - 16);    // the kernel keeps one iterate pointer per level, at most 16
  if (ls >= nl) return GLGPU_OK; // no smoothing level small enough
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int per_sm = vcycle_small_blocks_per_sm(c->mixed);
  if (per_sm < 1 || sms < 1) return GLGPU_OK;
  c->small_grid = sms * per_sm;
  return c->mixed ? small_setup_t<float>(c, ls) : small_setup_t<double>(c, ls);
}

// a grid barrier of the fused small-level V-cycle gave up waiting: clear its state and
// report the timeout
glgpu_status small_check(glgpu_ctx *c)
{
  if (!c->small_ls) return GLGPU_OK;
  int err = 0;
  CK(cudaMemcpyAsync(&err, c->small_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CKS(sync(c));
  if (!err) return GLGPU_OK;
  CK(cudaMemsetAsync(c->small_bar, 0, 2 * sizeof(unsigned int), c->st));
  CK(cudaMemsetAsync(c->small_err, 0, sizeof(int), c->st));
  CKS(sync(c));
  return set_error(GLGPU_ERR_TIMEOUT, "multigrid: a grid barrier of the fused coarse-level cycle timed out");
}

// The V-cycle's tail in one cluster launch per instance: the smoothing levels whose
// instances have at most kTailNodes nodes each (FP32/FP64 blocks), the dense level below
// them, and their parent, the finest level outside the tail.
constexpr int64_t kTailNodes = 160;
constexpr int kTailMaxLevels = 8; // smoothing levels the kernel walks

template <typename T> glgpu_status tail_setup_t(glgpu_ctx *c, int lp)
{
  const int nl = c->n_levels;
  std::vector<SmallLevel<T>> lev(static_cast<size_t>(nl - lp + 1));
  for (int l = lp; l <= nl; ++l)
    {
      glgpu_ctx *L = (l == 0) ? c : c->lv[l - 1];
      SmallLevel<T> &d = lev[static_cast<size_t>(l - lp)];
      d.m = L->dm;
      const bool smoothing = l > lp && l < nl; // the parent and the dense level only transfer
      d.vals = smoothing ? static_cast<const T *>(L->vals) : nullptr;
      d.dinv = smoothing ? static_cast<const T *>(L->dinv) : nullptr;
      d.r = static_cast<T *>(L->Bv);
      d.z = static_cast<T *>(L->X);
      d.t = static_cast<T *>(L->Tmp);
      d.t2 = static_cast<T *>(L->C1);
      if (l < nl)
        {
          const glgpu_ctx::Transfer &t = c->tr[l];
          d.r_ptr = t.r_ptr;
          d.r_idx = t.r_idx;
          d.r_w = static_cast<const T *>(t.r_w);
          d.p_ptr = t.p_ptr;
          d.p_idx = t.p_idx;
          d.p_w = static_cast<const T *>(t.p_w);
        }
    }
  std::vector<unsigned char> bytes(sizeof(SmallLevel<T>) * lev.size());
  std::memcpy(bytes.data(), lev.data(), bytes.size());
  unsigned char *dl = nullptr;
  CKS(dupload(c, &dl, bytes));
  c->tail_levels = dl;
  TailCycle<T> cy{};
  cy.n_tail = nl - lp - 1;
  cy.pre = std::max(1, c->prm[0].mg_pre);
  cy.post = std::max(0, c->prm[0].mg_post);
  cy.omega = static_cast<T>(c->prm[0].mg_omega);
  cy.dense_off = c->d_dense_off;
  cy.inv = c->d_inv;
  c->tail_cycle.resize(sizeof(cy));
  std::memcpy(c->tail_cycle.data(), &cy, sizeof(cy));
  c->tail_ls = lp + 1;
  return GLGPU_OK;
}

glgpu_status tail_setup(glgpu_ctx *c)
{
  const int nl = c->n_levels;
  if (nl < 2 || c->B != 18 || c->prm[0].mg_small_fuse != 2) return GLGPU_OK;
  int ls = nl; // first tail level
  while (ls - 1 >= 1)
    {
      const glgpu_ctx *L = c->lv[ls - 2]; // level ls - 1
      int64_t most = 0;
      for (int k = 0; k < c->n_inst; ++k) most = std::max(most, L->P.node_off[k + 1] - L->P.node_off[k]);
      if (most > kTailNodes || L->dm.half_vals || L->B != 18) break;
      --ls;
    }
  ls = std::max(ls, nl - kTailMaxLevels);
  if (ls >= nl) return GLGPU_OK; // no smoothing level small enough
  const int cs = vcycle_tail_cluster(c->mixed, c->n_inst);
  if (cs < 1) return GLGPU_OK;   // too many instances for clusters of useful size
  c->tail_cs = cs;
  return c->mixed ? tail_setup_t<float>(c, ls - 1) : tail_setup_t<double>(c, ls - 1);
}

glgpu_status mg_setup(glgpu_ctx *c, const glgpu_mesh *mesh, const glgpu_params *prm, int n_inst)
{
  std::vector<MgLevel> lv;
  std::string why;
  const int nl = build_hierarchy(mesh, n_inst, 16, lv, why);
  if (nl == 0) return GLGPU_OK; // multigrid does not apply: block-Jacobi stays in charge
  // coarse contexts share this context's stream
  std::vector<glgpu_params> lp(prm, prm + n_inst);
  for (auto &q : lp)
    {
      q.precond = GLGPU_PC_BLOCK_JACOBI;
      q.gmres_restart = 1;
      q.bt = 1e10; // coarse operators are Galerkin products of the fine one, Robin term included
    }
  for (int l = 0; l < nl; ++l)
    {
      std::vector<glgpu_mesh> ms(n_inst);
      for (int k = 0; k < n_inst; ++k)
        {
          const BoxMesh &b = lv[l].meshes[k];
          const bool con = !b.hpar.empty(); // periodic images
          ms[k] = glgpu_mesh{3, b.nn, b.nc, b.xyz.data(), b.cells.data(), b.mask.data(),
                             con ? b.hptr.data() : nullptr, con ? b.hpar.data() : nullptr, con ? b.hw.data() : nullptr};
        }
      glgpu_ctx *L = nullptr;
      glgpu_status st = glgpu_create(ms.data(), lp.data(), n_inst, &L);
      if (st != GLGPU_OK) return st;
      cudaStreamSynchronize(L->st);
      cudaStreamDestroy(L->st);
      L->st = c->st;
      L->owns_stream = false;
      L->mf = false; // coarse operators exist only assembled (Galerkin products)
      // in mixed mode the large coarse operators are stored in FP16: they serve only the
      // preconditioner of the flexible GMRES, and are swept twice per V-cycle at full bandwidth.
      // Small levels (latency-bound, and with the largest cells, whose mass-like entries grow
      // with the cell volume toward FP16's 65504) stay FP32.
      L->dm.half_vals = (c->mixed && L->nn >= 2000) ? 1 : 0;
      c->lv.push_back(L);
    }
  // transfer operators between level l (fine side) and l+1, and the Galerkin slot tables
  c->tr.resize(nl);
  for (int l = 0; l < nl; ++l)
    {
      const Plan &FP = (l == 0) ? c->P : c->lv[l - 1]->P;
      TransferTables T;
      // mixed mode keeps the Galerkin term weights in FP32: written so by the term pass
      glgpu_status ts = transfer_tables(mesh, n_inst, lv, l, FP, c->lv[l]->P, T, c->mixed);
      if (ts != GLGPU_OK) return ts;
      const std::vector<int32_t> &pp = T.pp, &pi = T.pi, &rp = T.rp, &ri = T.ri, &grow = T.g_row;
      const std::vector<double> &pw = T.pw, &rw = T.rw;
      const bulk_vector<int32_t> &gb = T.g_blk;
      const std::vector<int64_t> &gt = T.g_toff;
      glgpu_ctx::Transfer &t = c->tr[l];
      t.h_ptr = pp;
      t.h_idx = pi;
      t.h_w = pw;
      CKS(dupload(c, &t.p_ptr, pp));
      CKS(dupload(c, &t.p_idx, pi));
      CKS(dupload(c, &t.r_ptr, rp));
      CKS(dupload(c, &t.r_idx, ri));
      CKS(dupload(c, &t.g_toff, gt));
      CKS(dupload(c, &t.g_row, grow));
      CKS(dupload(c, &t.g_blk, gb));
      CKS(dupload(c, &t.g_up, T.g_up));
      CKS(dupload(c, &t.g_lo, T.g_lo));
      t.n_up = static_cast<int64_t>(T.g_up.size());
      t.n_lo = static_cast<int64_t>(T.g_lo.size() / 2);
      if (c->mixed)
        {
          CKS(upload_w<float>(c, &t.p_w, pw));
          CKS(upload_w<float>(c, &t.r_w, rw));
          float *gp = nullptr;
          CKS(dupload(c, &gp, T.g_wf));
          t.g_w = gp;
        }
      else
        {
          CKS(upload_w<double>(c, &t.p_w, pw));
          CKS(upload_w<double>(c, &t.r_w, rw));
          double *gp = nullptr;
          CKS(dupload(c, &gp, T.g_w));
          t.g_w = gp;
        }
      // fixed-slot copies of the two transfers (rows with more entries than slots keep the lists)
      auto slots = [&](const std::vector<int32_t> &ptr, const std::vector<int32_t> &idx, const std::vector<double> &w,
                       int S, TransferSlots &out) -> glgpu_status {
        const int64_t rows = static_cast<int64_t>(ptr.size()) - 1;
        for (int64_t r = 0; r < rows; ++r)
          if (ptr[r + 1] - ptr[r] > S) return GLGPU_OK;
        std::vector<int32_t> si(static_cast<size_t>(rows) * S, -1);
        std::vector<double> sw(static_cast<size_t>(rows) * S, 0.0);
        for (int64_t r = 0; r < rows; ++r)
          for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k)
            {
              si[static_cast<size_t>(r) * S + (k - ptr[r])] = idx[k];
              sw[static_cast<size_t>(r) * S + (k - ptr[r])] = w[k];
            }
        int32_t *d_si = nullptr;
        void *d_sw = nullptr;
        CKS(dupload(c, &d_si, si));
        if (c->mixed)
          CKS(upload_w<float>(c, &d_sw, sw));
        else
          CKS(upload_w<double>(c, &d_sw, sw));
        out.idx = d_si;
        out.w = d_sw;
        return GLGPU_OK;
      };
      CKS(slots(pp, pi, pw, kProlongSlots, t.p_slots));
      CKS(slots(rp, ri, rw, kRestrictSlots, t.r_slots));
    }
  // coarsest level: dense inverses
  glgpu_ctx *Lc = c->lv[nl - 1];
  std::vector<int64_t> doff(n_inst + 1, 0);
  int max_nd = 0;
  for (int k = 0; k < n_inst; ++k)
    {
      const int nd = static_cast<int>((Lc->P.node_off[k + 1] - Lc->P.node_off[k]) * Lc->B);
      max_nd = std::max(max_nd, nd);
      doff[k + 1] = doff[k] + static_cast<int64_t>(nd) * nd;
    }
  if (max_nd > 144) return set_error(GLGPU_ERR_ARG, "multigrid: coarsest level too large for the dense solve (144 unknowns)");
  c->max_nd = max_nd;
  {
    // the finest level's smoother blocks are read twice per V-cycle (the sweep from zero and
    // the post-sweep); with the matrix-free operator they are the largest array the cycle
    // reads there, so mixed mode stores them in FP16
    c->sinv_half = c->mixed && c->mf && c->B == 18;
    char *si = nullptr;
    CKS(dalloc(c, &si, (c->sinv_half ? sizeof(__half) : tsz(c)) * static_cast<size_t>(c->nn) * c->B * c->B));
    c->sinv = si;
    char *a = nullptr, *b = nullptr;
    CKS(dalloc(c, &a, tsz(c) * static_cast<size_t>(c->N)));
    CKS(dalloc(c, &b, tsz(c) * static_cast<size_t>(c->N)));
    CK(cudaMemset(a, 0, tsz(c) * static_cast<size_t>(c->N)));
    CK(cudaMemset(b, 0, tsz(c) * static_cast<size_t>(c->N)));
    c->mg_in = a;
    c->mg_out = b;
  }
  CKS(dupload(c, &c->d_dense_off, doff));
  CKS(dalloc(c, &c->d_inv, static_cast<size_t>(doff[n_inst])));
  CKS(dalloc(c, &c->d_sing, static_cast<size_t>(n_inst)));
  CK(cudaMemset(c->d_sing, 0, sizeof(int) * n_inst));
  {
    char *zb = nullptr;
    CKS(dalloc(c, &zb, tsz(c) * static_cast<size_t>(c->restart) * c->N));
    CK(cudaMemset(zb, 0, tsz(c) * static_cast<size_t>(c->restart) * c->N));
    c->Zb = zb;
  }
  c->n_levels = nl;
  CKS(small_setup(c));
  CKS(tail_setup(c));
  return GLGPU_OK;
}

} // namespace

// =================================================================================
// C ABI
// =================================================================================
extern "C" void glgpu_default_params(glgpu_params *p)
{
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->K1 = p->K2 = p->K3 = 0.42072;
  p->alpha = 0.0;
  p->precision = GLGPU_FP64;
  p->precond = GLGPU_PC_BLOCK_JACOBI;
  p->cheb_degree = 3;
  p->gmres_restart = 50;
  p->gmres_max_iter = 10000;
  p->ls_step = 0.83;
  p->ls_max_trials = 100;
  p->damped = 1;
  p->mg_pre = 1;
  p->mg_post = 1;
  p->mg_omega = 1.0;
  p->mf_cells = 8;
  p->prec_reuse = 0.0;
  p->bt = 1e10;
  p->mg_coarse_shift = 1e-4;
  p->mg_small_fuse = 0;
}

extern "C" const char *glgpu_version(void) { return "glgpu 0.1 (sm_103a)"; }

extern "C" const char *glgpu_last_error(void) { return g_last_error.c_str(); }

extern "C" glgpu_status glgpu_create(const glgpu_mesh *mesh, const glgpu_params *prm, int n_inst, glgpu_ctx **out)
{
  if (!out || !prm) return set_error(GLGPU_ERR_ARG, "glgpu_create: NULL argument");
  *out = nullptr;
  for (int k = 0; k < n_inst; ++k)
    {
      if (prm[k].precision != prm[0].precision || prm[k].precond != prm[0].precond ||
          prm[k].gmres_restart != prm[0].gmres_restart || prm[k].mf_cells != prm[0].mf_cells)
        return set_error(GLGPU_ERR_ARG,
                         "glgpu_create: precision, preconditioner, restart and mf_cells must match across instances");
    }
  for (int k = 0; k < n_inst; ++k)
    if (!(prm[k].bt > 0.0)) return set_error(GLGPU_ERR_ARG, "glgpu_create: bt (AdGR diffuse length) must be > 0");
  for (int k = 0; k < n_inst; ++k)
    if (!(prm[k].mg_coarse_shift > 0.0)) return set_error(GLGPU_ERR_ARG, "glgpu_create: mg_coarse_shift must be > 0");
  for (int k = 0; k < n_inst; ++k)
    if (prm[k].mg_small_fuse < 0 || prm[k].mg_small_fuse > 2)
      return set_error(GLGPU_ERR_ARG, "glgpu_create: mg_small_fuse must be 0, 1 or 2");
  if (prm[0].gmres_restart < 1 || prm[0].gmres_restart > 64)
    return set_error(GLGPU_ERR_ARG, "glgpu_create: gmres_restart must be in [1, 64]");
  if (prm[0].mf_cells != 4 && prm[0].mf_cells != 8 && prm[0].mf_cells != 16)
    return set_error(GLGPU_ERR_ARG, "glgpu_create: mf_cells must be 4, 8 or 16");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return set_error(GLGPU_ERR_CUDA, "glgpu_create: no CUDA device");
  glgpu_ctx *c = new glgpu_ctx();
  glgpu_status s = build_plan(mesh, n_inst, c->P);
  if (s != GLGPU_OK)
    {
      delete c;
      return s;
    }
  auto fail = [&](glgpu_status st) {
    std::string msg = g_last_error;
    glgpu_destroy(c);
    g_last_error = msg;
    return st;
  };
  const Plan &P = c->P;
  c->prm.assign(prm, prm + n_inst);
  c->B = P.B;
  c->n_inst = n_inst;
  c->nn = P.nn;
  c->N = P.nn * P.B;
  c->nnzb = P.nnzb;
  c->nq = (P.dim == 3) ? 8 : 4;
  c->ns = (P.dim == 3) ? kNS3 : 3;
  c->mixed = prm[0].precision == GLGPU_MIXED;
  c->restart = prm[0].gmres_restart;
  if (P.dim == 3 && static_cast<size_t>(P.max_row_blocks) * 324 * (c->mixed ? 4 : 8) > 220 * 1024)
    return fail(set_error(GLGPU_ERR_ARG, "glgpu_create: a block row is too long for on-chip accumulation"));
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess)
    return fail(set_error(GLGPU_ERR_CUDA, "glgpu_create: stream creation failed"));
  if (init_constants() != cudaSuccess) return fail(set_error(GLGPU_ERR_CUDA, "glgpu_create: constant upload failed"));
  DevMesh &d = c->dm;
  d.dim = P.dim;
  d.B = P.B;
  d.nv = P.nv;
  d.n_inst = n_inst;
  d.nn = P.nn;
  d.nc = P.nc;
  d.nnzb = P.nnzb;
  d.max_row_blocks = P.max_row_blocks;
  int32_t *p_cells, *p_ci, *p_ni, *p_hptr, *p_hpar, *p_rowptr, *p_cols, *p_diag, *p_rcp, *p_rcc, *p_rca, *p_si, *p_iso;
  uint32_t *p_mask;
  double *p_h, *p_hw, *p_rcw, *p_coef;
  int16_t *p_slot;
  int64_t *p_hto, *p_sb, *p_se, *p_co, *p_noff;
  HangTarget *p_tg;
  std::vector<double> coef(static_cast<size_t>(n_inst) * kCoef);
  std::vector<GeoD> geo_d(P.nc);
  std::vector<float4> geo_f(P.nc);
  for (int64_t e = 0; e < P.nc; ++e)
    {
      const double hx = P.cell_h[3 * e], hy = P.cell_h[3 * e + 1], hz = P.cell_h[3 * e + 2];
      geo_d[e] = GeoD{1.0 / hx, 1.0 / hy, 1.0 / hz, hx * hy * hz};
      geo_f[e] = make_float4(static_cast<float>(1.0 / hx), static_cast<float>(1.0 / hy), static_cast<float>(1.0 / hz),
                             static_cast<float>(hx * hy * hz));
    }
  std::vector<float> rc_wf(P.rc_w.begin(), P.rc_w.end());
  GeoD *p_geod;
  float4 *p_geof;
  float *p_coeff, *p_rcwf;
  for (int k = 0; k < n_inst; ++k)
    {
      coef[k * kCoef + 0] = prm[k].K1;
      coef[k * kCoef + 1] = prm[k].K2 + prm[k].K3;
      coef[k * kCoef + 2] = prm[k].alpha;
      for (int t = 0; t < 5; ++t) coef[k * kCoef + 3 + t] = prm[k].beta[t];
      coef[k * kCoef + 8] = (prm[k].bt < 1e10) ? prm[k].K1 / prm[k].bt : 0.0; // assemble.cc:292
    }
  if ((s = dupload(c, &p_cells, P.cells)) || (s = dupload(c, &p_h, P.cell_h)) || (s = dupload(c, &p_ci, P.cell_inst)) ||
      (s = dupload(c, &p_ni, P.node_inst)) || (s = dupload(c, &p_mask, P.mask)) || (s = dupload(c, &p_hptr, P.hptr)) ||
      (s = dupload(c, &p_hpar, P.hpar)) || (s = dupload(c, &p_hw, P.hw)) || (s = dupload(c, &p_rowptr, P.rowptr)) ||
      (s = dupload(c, &p_cols, P.cols)) || (s = dupload(c, &p_diag, P.diag)) || (s = dupload(c, &p_rcp, P.rc_ptr)) ||
      (s = dupload(c, &p_rcc, P.rc_cell)) || (s = dupload(c, &p_rca, P.rc_a)) || (s = dupload(c, &p_rcw, P.rc_w)) ||
      (s = dupload(c, &p_slot, P.rc_slot)) || (s = dupload(c, &p_hto, P.ht_off)) || (s = dupload(c, &p_tg, P.hang_tg)) ||
      (s = dupload(c, &p_coef, coef)) || (s = dupload(c, &p_sb, P.seg_begin)) || (s = dupload(c, &p_se, P.seg_end)) ||
      (s = dupload(c, &p_si, P.seg_inst)) || (s = dupload(c, &p_iso, P.inst_seg_off)) ||
      (s = dupload(c, &p_co, P.cell_off)) || (s = dupload(c, &p_noff, P.node_off)) ||
      (s = dupload(c, &p_geod, geo_d)) || (s = dupload(c, &p_geof, geo_f)) ||
      (s = dupload(c, &p_rcwf, rc_wf)))
    return fail(s);
  {
    int32_t *p_reg = nullptr, *p_gen = nullptr;
    if ((s = dupload(c, &p_reg, P.reg_rows)) || (s = dupload(c, &p_gen, P.gen_rows))) return fail(s);
    d.reg_rows = p_reg;
    d.gen_rows = p_gen;
    d.n_reg = static_cast<int64_t>(P.reg_rows.size());
    d.n_gen = static_cast<int64_t>(P.gen_rows.size());
    // gradient part of the interior rows of every instance with cells of one size
    std::vector<double> tmpl(static_cast<size_t>(n_inst) * 27 * 324, 0.0);
    if (P.dim == 3 && P.B == 18)
      for (int k = 0; k < n_inst; ++k)
        if (P.inst_uniform[k])
          regular_row_stiffness(prm[k].K1, prm[k].K2 + prm[k].K3, &P.inst_h[3 * k], &tmpl[static_cast<size_t>(k) * 27 * 324]);
    std::vector<float> tmpl_f(tmpl.begin(), tmpl.end());
    double *p_td = nullptr;
    float *p_tf = nullptr;
    if ((s = dupload(c, &p_td, tmpl)) || (s = dupload(c, &p_tf, tmpl_f))) return fail(s);
    d.reg_tmpl_d = p_td;
    d.reg_tmpl_f = p_tf;
  }
  {
    // Robin faces of the instances with bt < 1e10
    std::vector<uint8_t> on(n_inst, 0), robin;
    for (int k = 0; k < n_inst; ++k) on[k] = (P.dim == 3 && P.B == 18 && prm[k].bt < 1e10) ? 1 : 0;
    robin_faces(P, on, robin);
    std::vector<int32_t> rcells;
    for (int64_t e = 0; e < P.nc; ++e)
      if (robin[e]) rcells.push_back(static_cast<int32_t>(e));
    d.robin = nullptr;
    d.robin_cells = nullptr;
    d.n_robin = static_cast<int64_t>(rcells.size());
    if (!rcells.empty())
      {
        uint8_t *p_rb = nullptr;
        int32_t *p_rc = nullptr;
        if ((s = dupload(c, &p_rb, robin)) || (s = dupload(c, &p_rc, rcells))) return fail(s);
        d.robin = p_rb;
        d.robin_cells = p_rc;
      }
  }
  {
    std::vector<float> cf(coef.begin(), coef.end());
    if ((s = dupload(c, &p_coeff, cf))) return fail(s);
  }
  d.geo_d = p_geod;
  d.geo_f = p_geof;
  d.coef_f = p_coeff;
  d.rc_wf = p_rcwf;
  d.cells = p_cells;
  d.cell_h = p_h;
  d.cell_inst = p_ci;
  d.node_inst = p_ni;
  d.mask = p_mask;
  d.hptr = p_hptr;
  d.has_constraints = (!P.hptr.empty() && P.hptr.back() > 0) ? 1 : 0;
  {
    // the matrix-free gather's contribution table: on meshes without constraint rows every
    // node takes at most 8 cell contributions, all of weight 1; rc_off8[n][k] is the offset
    // cell * 144 + vertex * 18 of its k-th contribution in list order, -1 past the end
    int32_t *p_off8 = nullptr;
    if (P.dim == 3 && P.B == 18 && P.nv == 8 && !d.has_constraints && P.nc * 144 < INT32_MAX)
      {
        bool ok = true;
        std::vector<int32_t> off8(static_cast<size_t>(P.nn) * 8, -1);
        for (int64_t n = 0; n < P.nn && ok; ++n)
          {
            const int32_t k0 = P.rc_ptr[n], k1 = P.rc_ptr[n + 1];
            ok = k1 - k0 <= 8;
            for (int32_t k = k0; ok && k < k1; ++k)
              {
                ok = P.rc_w[k] == 1.0;
                off8[static_cast<size_t>(n) * 8 + (k - k0)] = static_cast<int32_t>(P.rc_cell[k] * 144 + P.rc_a[k] * 18);
              }
          }
        if (ok && (s = dupload(c, &p_off8, off8))) return fail(s);
        if (!ok) p_off8 = nullptr;
      }
    d.rc_off8 = p_off8;
  }
  {
    int32_t *p_c27 = nullptr;
    if (P.B == 18 && P.max_row_blocks <= 27)
      {
        std::vector<int32_t> c27(static_cast<size_t>(P.nn) * 27, -1);
        for (int64_t n = 0; n < P.nn; ++n)
          for (int32_t b = P.rowptr[n]; b < P.rowptr[n + 1]; ++b)
            c27[static_cast<size_t>(n) * 27 + (b - P.rowptr[n])] = P.cols[b];
        if ((s = dupload(c, &p_c27, c27))) return fail(s);
      }
    d.cols27 = p_c27;
  }
  d.hpar = p_hpar;
  d.hw = p_hw;
  d.rowptr = p_rowptr;
  d.cols = p_cols;
  d.diag = p_diag;
  d.rc_ptr = p_rcp;
  d.rc_cell = p_rcc;
  d.rc_a = p_rca;
  d.rc_w = p_rcw;
  d.rc_slot = p_slot;
  d.ht_off = p_hto;
  d.hang_tg = p_tg;
  d.coef = p_coef;
  d.n_seg = static_cast<int>(P.seg_begin.size());
  d.seg_begin = p_sb;
  d.seg_end = p_se;
  d.seg_inst = p_si;
  d.inst_seg_off = p_iso;
  d.cell_off = p_co;
  d.node_off_ptr = p_noff;
  // state buffers
  const int64_t N = c->N;
  const size_t ts = tsz(c);
  const int mr = c->restart;
  const int deg = std::max(1, prm[0].cheb_degree);
  void *pv;
  if ((s = dalloc(c, &c->x, N)) || (s = dalloc(c, &c->xt, N)) || (s = dalloc(c, &c->delta, N)) ||
      (s = dalloc(c, &c->R, N)) || (s = dalloc(c, &c->rhs, N)) ||
      (s = dalloc(c, &c->r_cell, static_cast<size_t>(P.nc) * P.nv * P.B)) || (s = dalloc(c, &c->e_cell, P.nc)))
    return fail(s);
  auto talloc = [&](void **p, size_t count) -> glgpu_status {
    char *q = nullptr;
    glgpu_status st = dalloc(c, &q, count * ts);
    *p = q;
    return st;
  };
  if ((s = talloc(&c->H, static_cast<size_t>(P.nc) * c->nq * c->ns)) ||
      (s = talloc(&c->vals, static_cast<size_t>(P.nnzb) * P.B * P.B)) ||
      (s = talloc(&c->dinv, static_cast<size_t>(P.nn) * P.B * P.B)) ||
      (s = talloc(&c->V, static_cast<size_t>(mr + 1) * N)) || (s = talloc(&c->Z, N)) || (s = talloc(&c->X, N)) ||
      (s = talloc(&c->Tmp, N)) || (s = talloc(&c->Bv, N)) || (s = talloc(&c->C1, N)) || (s = talloc(&c->C2, N)) ||
      (s = talloc(&c->C3, N)))
    return fail(s);
  (void)pv;
  // mixed 3D contexts apply the Krylov operator matrix-free at the state
  if (c->mixed && P.dim == 3 && P.B == 18 && P.nv == 8)
    {
      if ((s = dalloc(c, &c->ycell, static_cast<size_t>(P.nc) * P.nv * P.B)) ||
          (s = dalloc(c, &c->x32, static_cast<size_t>(c->N))))
        return fail(s);
      c->mf = true;
    }
  if ((s = dalloc(c, &c->partial, static_cast<size_t>(d.n_seg) * (mr + 2))) ||
      (s = dalloc(c, &c->partial_n, static_cast<size_t>(d.n_seg))) ||
      (s = dalloc(c, &c->g.H, static_cast<size_t>(n_inst) * (mr + 1) * mr)) ||
      (s = dalloc(c, &c->g.cs, static_cast<size_t>(n_inst) * mr)) ||
      (s = dalloc(c, &c->g.sn, static_cast<size_t>(n_inst) * mr)) ||
      (s = dalloc(c, &c->g.g, static_cast<size_t>(n_inst) * (mr + 1))) ||
      (s = dalloc(c, &c->g.y, static_cast<size_t>(n_inst) * mr)) ||
      (s = dalloc(c, &c->g.hcol, static_cast<size_t>(n_inst) * (mr + 2))) ||
      (s = dalloc(c, &c->g.hcol2, static_cast<size_t>(n_inst) * (mr + 2))) || (s = dalloc(c, &c->g.beta, n_inst)) ||
      (s = dalloc(c, &c->g.tol, n_inst)) || (s = dalloc(c, &c->g.res_est, n_inst)) ||
      (s = dalloc(c, &c->g.its, n_inst)) || (s = dalloc(c, &c->g.active, n_inst)) ||
      (s = dalloc(c, &c->g.inv_scale, n_inst)) || (s = dalloc(c, &c->d_norm, n_inst)) ||
      (s = dalloc(c, &c->d_a, n_inst)) || (s = dalloc(c, &c->d_energy, n_inst)) ||
      (s = dalloc(c, &c->d_tmp, n_inst)) ||
      (s = dalloc(c, &c->d_cheb, static_cast<size_t>(n_inst) * 2 * (deg + 1))) || (s = dalloc(c, &c->d_act, n_inst)) ||
      (s = dalloc(c, &c->d_act2, n_inst)) || (s = dalloc(c, &c->d_cnt, n_inst)))
    return fail(s);
  if (cudaMemset(c->d_cnt, 0, sizeof(unsigned int) * n_inst) != cudaSuccess)
    return fail(set_error(GLGPU_ERR_CUDA, "glgpu_create: counter initialisation failed"));
  c->g.m = mr;
  if (cudaMallocHost(&c->h_norm, sizeof(double) * std::max(n_inst, 2 * n_inst * (deg + 1))) != cudaSuccess ||
      cudaMallocHost(&c->h_res, sizeof(double) * std::max(n_inst, 2 * n_inst * (deg + 1))) != cudaSuccess ||
      cudaMallocHost(&c->h_act, n_inst) != cudaSuccess || cudaMallocHost(&c->h_act_pipe, 2 * n_inst) != cudaSuccess ||
      cudaMallocHost(&c->h_its, sizeof(int) * n_inst) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_pipe[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_pipe[1], cudaEventDisableTiming) != cudaSuccess)
    return fail(set_error(GLGPU_ERR_NOMEM, "glgpu_create: pinned host allocation failed"));
  if (cudaMemsetAsync(c->x, 0, sizeof(double) * N, c->st) != cudaSuccess ||
      cudaMemsetAsync(c->delta, 0, sizeof(double) * N, c->st) != cudaSuccess ||
      cudaMemsetAsync(c->R, 0, sizeof(double) * N, c->st) != cudaSuccess ||
      cudaMemsetAsync(c->rhs, 0, sizeof(double) * N, c->st) != cudaSuccess ||
      cudaMemsetAsync(c->V, 0, tsz(c) * static_cast<size_t>(mr + 1) * N, c->st) != cudaSuccess ||
      cudaMemsetAsync(c->H, 0, tsz(c) * static_cast<size_t>(P.nc) * c->nq * c->ns, c->st) != cudaSuccess ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    return fail(set_error(GLGPU_ERR_CUDA, "glgpu_create: initialisation failed"));
  c->rhs_norm.assign(n_inst, 0.0);
  c->res_norm.assign(n_inst, 0.0);
  c->inst_on.assign(n_inst, 1);
  c->handed.assign(n_inst, 0);
  c->r_ok.assign(n_inst, 0);
  c->stop_ls.assign(n_inst, 0.0);
  c->stop_fp64.assign(n_inst, 0.0);
  cudaEventCreate(&c->ev_user0);
  cudaEventCreate(&c->ev_user1);
  if (prm[0].precond == GLGPU_PC_MULTIGRID && P.dim == 3)
    {
      if ((s = mg_setup(c, mesh, prm, n_inst)) != GLGPU_OK) return fail(s);
    }
  *out = c;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_destroy(glgpu_ctx *c)
{
  if (!c) return GLGPU_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  for (auto &r : c->kev)
    {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
  for (auto &r : c->pev)
    {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  if (c->ev_user0) cudaEventDestroy(c->ev_user0);
  if (c->ev_user1) cudaEventDestroy(c->ev_user1);
  for (void *p : c->allocs) cudaFree(p);
  if (c->h_norm) cudaFreeHost(c->h_norm);
  if (c->h_res) cudaFreeHost(c->h_res);
  if (c->h_act) cudaFreeHost(c->h_act);
  if (c->h_act_pipe) cudaFreeHost(c->h_act_pipe);
  for (auto e : c->ev_pipe)
    if (e) cudaEventDestroy(e);
  if (c->h_its) cudaFreeHost(c->h_its);
  if (c->vc_exec) cudaGraphExecDestroy(c->vc_exec);
  for (glgpu_ctx *l : c->lv) glgpu_destroy(l);
  if (c->st && c->owns_stream) cudaStreamDestroy(c->st);
  delete c;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_sizes(const glgpu_ctx *c, int64_t *n_nodes, int64_t *nnzb, int *block, int *n_inst)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_sizes: NULL context");
  if (n_nodes) *n_nodes = c->nn;
  if (nnzb) *nnzb = c->nnzb;
  if (block) *block = c->B;
  if (n_inst) *n_inst = c->n_inst;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_set_solution(glgpu_ctx *c, const double *x)
{
  if (!c || !x) return set_error(GLGPU_ERR_ARG, "glgpu_set_solution: NULL argument");
  CK(cudaMemcpyAsync(c->x, x, sizeof(double) * c->N, cudaMemcpyHostToDevice, c->st));
  CK(launch_distribute(c->dm, c->x, c->st));
  c->launches += 2;
  c->has_J = c->has_rhs = c->has_delta = false;
  std::fill(c->r_ok.begin(), c->r_ok.end(), 0);
  c->prec_built = false;
  c->last_step_rel = 1e300;
  return sync(c);
}

extern "C" glgpu_status glgpu_host_alloc(size_t bytes, void **p)
{
  if (!p) return set_error(GLGPU_ERR_ARG, "glgpu_host_alloc: NULL argument");
  *p = nullptr;
  if (cudaMallocHost(p, bytes > 0 ? bytes : 1) != cudaSuccess)
    return set_error(GLGPU_ERR_NOMEM, "glgpu_host_alloc: cudaMallocHost failed");
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_host_free(void *p)
{
  if (p && cudaFreeHost(p) != cudaSuccess) return set_error(GLGPU_ERR_CUDA, "glgpu_host_free: cudaFreeHost failed");
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_get_solution(const glgpu_ctx *c, double *x)
{
  if (!c || !x) return set_error(GLGPU_ERR_ARG, "glgpu_get_solution: NULL argument");
  CK(cudaMemcpyAsync(x, c->x, sizeof(double) * c->N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return GLGPU_OK;
}

static glgpu_status assemble_impl(glgpu_ctx *c, const uint8_t *act)
{
  PhaseScope ps(c, PH_ASM);
  // the line search of the previous Newton step already evaluated R at the accepted
  // state (same kernels, same x): reuse it instead of recomputing the FP64 residual
  bool need_r = false;
  for (int k = 0; k < c->n_inst; ++k)
    if ((!act || c->inst_on[k]) && !c->r_ok[k]) need_r = true;
  if (!c->mixed)
    {
      CKS(launch(c, KK_CELL, 1, [&] {
        return launch_cell(c->dm, false, c->x, c->H, need_r ? c->r_cell : nullptr, need_r ? c->e_cell : nullptr, act,
                           c->st);
      }));
      if (need_r) CKS(robin_res(c, c->x, c->e_cell, act));
    }
  // a small last Newton step keeps the previous preconditioner; the matrix-free operator
  // works from the state alone, so the Hessians and the block matrix are then formed only
  // on demand
  const double reuse = c->prm[0].prec_reuse;
  const bool keep_prec = reuse > 0 && c->mf && c->n_levels > 0 && c->prec_built && c->last_step_rel < reuse;
  if (c->mixed)
    {
      if (c->mf) CKS(axpby(c, c->x, c->x32, nullptr, coefs(1.0, 0.0), act, false, true, true));
      if (!keep_prec)
        CKS(launch(c, KK_CELL, 1, [&] { return launch_cell(c->dm, true, c->x, c->H, nullptr, nullptr, act, c->st); }));
      if (need_r)
        {
          CKS(launch(c, KK_RES, 1, [&] {
            return launch_cell(c->dm, true, c->x, nullptr, c->r_cell, nullptr, act, c->st);
          }));
          CKS(robin_res(c, c->x, nullptr, act));
        }
    }
  if (keep_prec)
    c->bsr_stale = true;
  else
    {
      CKS(launch(c, KK_ROWS, 1, [&] { return launch_rows(c->dm, c->mixed, c->H, c->vals, c->st); }));
      c->bsr_stale = false;
    }
  if (need_r) CKS(launch(c, KK_RES, 1, [&] { return launch_res_gather(c->dm, c->r_cell, c->R, act, c->st); }));
  CKS(axpby(c, c->R, c->rhs, nullptr, coefs(-1.0, 0.0), act, false, false, false));
  std::vector<double> nr;
  CKS(norms_d(c, c->rhs, act, nr));
  for (int k = 0; k < c->n_inst; ++k)
    if (!act || c->inst_on[k]) c->rhs_norm[k] = nr[k];
  c->has_J = c->has_rhs = true;
  for (int k = 0; k < c->n_inst; ++k)
    if (!act || c->inst_on[k]) c->r_ok[k] = 1;
  if (!keep_prec) c->prec_ready = c->dinv_ready = false;
  for (int k = 0; k < c->n_inst; ++k)
    if ((!act || c->inst_on[k]) && !std::isfinite(c->rhs_norm[k]))
      return set_error(GLGPU_ERR_NAN, "assemble_system: non-finite residual in instance " + std::to_string(k));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_assemble_system(glgpu_ctx *c, double *rhs_norm)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_assemble_system: NULL context");
  std::fill(c->inst_on.begin(), c->inst_on.end(), 1);
  CKS(assemble_impl(c, nullptr));
  if (rhs_norm) std::copy(c->rhs_norm.begin(), c->rhs_norm.end(), rhs_norm);
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_compute_residual(glgpu_ctx *c, double *norm)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_compute_residual: NULL context");
  {
    PhaseScope ps(c, PH_RES);
    CKS(residual_at(c, c->x, nullptr));
    std::fill(c->r_ok.begin(), c->r_ok.end(), 1);
  }
  std::vector<double> nr;
  CKS(norms_d(c, c->R, nullptr, nr));
  c->res_norm = nr;
  if (norm) std::copy(nr.begin(), nr.end(), norm);
  for (double v : nr)
    if (!std::isfinite(v)) return set_error(GLGPU_ERR_NAN, "compute_residual: non-finite residual");
  return GLGPU_OK;
}

static glgpu_status solve_impl(glgpu_ctx *c, double tol, std::vector<int> &its, bool &conv)
{
  if (!c->has_J) return set_error(GLGPU_ERR_STATE, "solve: assemble_system must come first");
  PhaseScope ps(c, PH_SOLVE);
  bool all_on = true;
  for (int k = 0; k < c->n_inst; ++k) all_on &= c->inst_on[k] != 0;
  if (!all_on) CKS(upload_act(c, c->d_act, c->inst_on));
  CKS(prec_setup(c, all_on ? nullptr : c->d_act));
  CKS(gmres(c, tol, c->inst_on, its, conv));
  CKS(small_check(c));
  c->has_delta = true;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_solve(glgpu_ctx *c, double tol, int *its)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_solve: NULL context");
  std::vector<int> it;
  bool conv = false;
  CKS(solve_impl(c, tol, it, conv));
  if (its) std::copy(it.begin(), it.end(), its);
  if (!conv) return set_error(GLGPU_ERR_NOT_CONVERGED, "solve: GMRES reached the iteration limit");
  return GLGPU_OK;
}

static glgpu_status newton_impl(glgpu_ctx *c, std::vector<double> &res, std::vector<int> &trials)
{
  if (!c->has_delta || !c->has_rhs) return set_error(GLGPU_ERR_STATE, "newton_iteration: solve must come first");
  PhaseScope ps(c, PH_NEWTON);
  const int n = c->n_inst;
  const glgpu_params &p0 = c->prm[0];
  const int max_trials = p0.damped ? std::max(1, p0.ls_max_trials) : 1;
  std::vector<uint8_t> pending(c->inst_on);
  std::vector<double> cur(n, 0.0), a(n, 0.0);
  for (int k = 0; k < n; ++k)
    if (c->inst_on[k]) c->r_ok[k] = 0; // the trials overwrite R
  res.assign(n, 0.0);
  trials.assign(n, 0);
  for (int i = 0; i < max_trials; ++i)
    {
      bool any = false;
      for (int k = 0; k < n; ++k)
        if (pending[k])
          {
            any = true;
            a[k] = c->prm[k].damped ? std::pow(c->prm[k].ls_step, static_cast<double>(i)) : 1.0;
          }
      if (!any) break;
      CKS(upload_d(c, c->d_a, a));
      CKS(upload_act(c, c->d_act, pending));
      CKS(launch(c, KK_VEC, 1, [&] { return launch_trial(c->dm, c->x, c->delta, c->d_a, c->xt, c->d_act, c->st); }));
      CKS(residual_at(c, c->xt, c->d_act));
      std::vector<double> nr;
      CKS(norms_d(c, c->R, c->d_act, nr));
      for (int k = 0; k < n; ++k)
        if (pending[k])
          {
            cur[k] = nr[k];
            trials[k] = i + 1;
            if (nr[k] < c->rhs_norm[k] || !c->prm[k].damped) pending[k] = 0;
          }
    }
  // local_solution = the accepted (or last) trial
  CKS(upload_act(c, c->d_act, c->inst_on));
  CKS(axpby(c, c->xt, c->x, nullptr, coefs(1.0, 0.0), c->d_act, false, false, false));
  for (int k = 0; k < n; ++k)
    if (c->inst_on[k])
      {
        res[k] = cur[k];
        c->res_norm[k] = cur[k];
      }
  c->has_J = c->has_rhs = c->has_delta = false;
  // R, r_cell, e_cell now hold the values at the new x of every instance of the step
  for (int k = 0; k < n; ++k)
    if (c->inst_on[k]) c->r_ok[k] = 1;
  if (c->prm[0].prec_reuse > 0)
    {
      std::vector<double> nd, nx;
      CKS(norms_d(c, c->delta, c->d_act, nd));
      CKS(norms_d(c, c->x, c->d_act, nx));
      double rel = 0.0;
      for (int k = 0; k < n; ++k)
        if (c->inst_on[k]) rel = std::max(rel, (nx[k] > 0 ? a[k] * nd[k] / nx[k] : 1e300));
      c->last_step_rel = rel;
    }
  for (int k = 0; k < n; ++k)
    if (c->inst_on[k] && !std::isfinite(res[k]))
      return set_error(GLGPU_ERR_NAN, "newton_iteration: non-finite residual in instance " + std::to_string(k));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_newton_iteration(glgpu_ctx *c, double *res, int *trials)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_newton_iteration: NULL context");
  std::vector<double> r;
  std::vector<int> t;
  CKS(newton_impl(c, r, t));
  if (res) std::copy(r.begin(), r.end(), res);
  if (trials) std::copy(t.begin(), t.end(), trials);
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_free_energy(glgpu_ctx *c, double *F)
{
  if (!c || !F) return set_error(GLGPU_ERR_ARG, "glgpu_free_energy: NULL argument");
  CKS(residual_at(c, c->x, nullptr, true, true)); // FP64 in every precision mode
  std::fill(c->r_ok.begin(), c->r_ok.end(), 1);
  CKS(launch(c, KK_VEC, 1, [&] { return launch_cell_sum(c->dm, c->e_cell, c->d_energy, c->st); }));
  CK(cudaMemcpyAsync(c->h_norm, c->d_energy, sizeof(double) * c->n_inst, cudaMemcpyDeviceToHost, c->st));
  CKS(sync(c));
  std::copy(c->h_norm, c->h_norm + c->n_inst, F);
  return GLGPU_OK;
}

// ---------------------------------------------------------------------------------
// Kelly error estimator and refinement flags (refine.cc:147-157)
// ---------------------------------------------------------------------------------
namespace
{
glgpu_status kelly_setup(glgpu_ctx *c)
{
  glgpu_ctx::Kelly &K = c->kelly;
  if (K.ready) return GLGPU_OK;
  KellyFaces F;
  CKS(kelly_faces(c->P, F));
  K.np = static_cast<int64_t>(F.a.size());
  if (K.np > 0)
    {
      CKS(dupload(c, &K.a, F.a));
      CKS(dupload(c, &K.b, F.b));
      CKS(dupload(c, &K.fa, F.fa));
      CKS(dupload(c, &K.ob, F.ob));
      CKS(dupload(c, &K.sub, F.sub));
      CKS(dupload(c, &K.cpair, F.cell_pair));
      CKS(dalloc(c, &K.I, static_cast<size_t>(K.np)));
    }
  CKS(dupload(c, &K.cptr, F.cell_ptr));
  CKS(dalloc(c, &K.eta, static_cast<size_t>(c->P.nc)));
  CKS(dalloc(c, &K.flags, static_cast<size_t>(c->P.nc)));
  CKS(dalloc(c, &K.prefix, static_cast<size_t>(c->n_inst)));
  CKS(dalloc(c, &K.thr_r, static_cast<size_t>(c->n_inst)));
  CKS(dalloc(c, &K.thr_c, static_cast<size_t>(c->n_inst)));
  CKS(dalloc(c, &K.hist, static_cast<size_t>(c->n_inst) * 256));
  K.ready = true;
  return GLGPU_OK;
}

// bit patterns of the rank[k]-th largest estimate of every instance (rank >= 1), or
// 0xffffffff where rank[k] == 0
glgpu_status kelly_select(glgpu_ctx *c, const std::vector<int64_t> &rank, std::vector<uint32_t> &out)
{
  glgpu_ctx::Kelly &K = c->kelly;
  const int n = c->n_inst;
  std::vector<uint32_t> prefix(n, 0u), hist(static_cast<size_t>(n) * 256);
  std::vector<int64_t> r(rank);
  for (int shift = 24; shift >= 0; shift -= 8)
    {
      CK(cudaMemcpyAsync(K.prefix, prefix.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, c->st));
      CKS(launch(c, KK_VEC, 1, [&] { return launch_radix_hist(c->dm, K.eta, K.prefix, shift, K.hist, c->st); }));
      CK(cudaMemcpyAsync(hist.data(), K.hist, sizeof(uint32_t) * 256 * n, cudaMemcpyDeviceToHost, c->st));
      CKS(sync(c));
      for (int k = 0; k < n; ++k)
        {
          if (r[k] <= 0) continue;
          int64_t above = 0;
          for (int bin = 255; bin >= 0; --bin)
            {
              const int64_t h = hist[static_cast<size_t>(k) * 256 + bin];
              if (above + h >= r[k])
                {
                  prefix[k] |= static_cast<uint32_t>(bin) << shift;
                  r[k] -= above;
                  break;
                }
              above += h;
            }
        }
    }
  out.assign(n, 0xffffffffu);
  for (int k = 0; k < n; ++k)
    if (rank[k] > 0) out[k] = prefix[k];
  return GLGPU_OK;
}
} // namespace

extern "C" glgpu_status glgpu_estimate_error(glgpu_ctx *c, float *eta)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_estimate_error: NULL context");
  if (c->P.dim != 3 || c->B != 18) return set_error(GLGPU_ERR_ARG, "glgpu_estimate_error: 3D femgl contexts only");
  CKS(kelly_setup(c));
  glgpu_ctx::Kelly &K = c->kelly;
  CKS(launch(c, KK_VEC, K.np > 0 ? 2 : 1, [&] {
    return launch_kelly(c->dm, c->x, K.a, K.b, K.fa, K.ob, K.sub, K.np, K.cptr, K.cpair, K.I, K.eta, c->st);
  }));
  if (eta) CK(cudaMemcpyAsync(eta, K.eta, sizeof(float) * c->P.nc, cudaMemcpyDeviceToHost, c->st));
  CKS(sync(c));
  K.eta_valid = true;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_refine_flags(glgpu_ctx *c, double top_fraction, double bottom_fraction, int8_t *flags)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_refine_flags: NULL context");
  if (!(top_fraction >= 0.0 && bottom_fraction >= 0.0 && top_fraction + bottom_fraction <= 1.0))
    return set_error(GLGPU_ERR_ARG, "glgpu_refine_flags: need 0 <= fractions and top + bottom <= 1");
  if (!c->kelly.ready || !c->kelly.eta_valid)
    return set_error(GLGPU_ERR_STATE, "glgpu_refine_flags: call glgpu_estimate_error first");
  const int n = c->n_inst;
  std::vector<int64_t> rr(n), rc(n);
  for (int k = 0; k < n; ++k)
    {
      const int64_t nk = c->P.cell_off[k + 1] - c->P.cell_off[k];
      const int64_t kr = static_cast<int64_t>(top_fraction * static_cast<double>(nk));
      const int64_t kc = static_cast<int64_t>(bottom_fraction * static_cast<double>(nk));
      rr[k] = kr;
      rc[k] = kc > 0 ? nk - kc + 1 : 0; // the kc-th smallest is the (nk - kc + 1)-th largest
    }
  std::vector<uint32_t> tr, tc;
  CKS(kelly_select(c, rr, tr));
  CKS(kelly_select(c, rc, tc));
  glgpu_ctx::Kelly &K = c->kelly;
  CK(cudaMemcpyAsync(K.thr_r, tr.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(K.thr_c, tc.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, c->st));
  CKS(launch(c, KK_VEC, 1, [&] { return launch_flags(c->dm, K.eta, K.thr_r, K.thr_c, K.flags, c->st); }));
  if (flags) CK(cudaMemcpyAsync(flags, K.flags, sizeof(int8_t) * c->P.nc, cudaMemcpyDeviceToHost, c->st));
  CKS(sync(c));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_run(glgpu_ctx *c, int max_newton, double linear_tol, double converge_acc,
                                  int *newton_its, int *gmres_its, double *final_res)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_run: NULL context");
  const int n = c->n_inst;
  std::vector<int> nits(n, 0), gits(n, 0);
  std::vector<double> fres(n, 0.0);
  std::fill(c->inst_on.begin(), c->inst_on.end(), 1);
  std::fill(c->handed.begin(), c->handed.end(), 0);
  glgpu_status result = GLGPU_OK;
  for (int it = 0; it <= max_newton; ++it)
    {
      CKS(upload_act(c, c->d_act, c->inst_on));
      CKS(assemble_impl(c, c->d_act));
      std::vector<int> its;
      bool conv = false;
      CKS(solve_impl(c, linear_tol, its, conv));
      bool any_on = false;
      for (int k = 0; k < n; ++k)
        if (c->inst_on[k] && c->handed[k])
          {
            // handed off: keep the state, count the linear iterations spent
            c->inst_on[k] = 0;
            gits[k] += its[k];
          }
        else
          any_on |= c->inst_on[k] != 0;
      if (!any_on) break;
      std::vector<double> r;
      std::vector<int> t;
      CKS(newton_impl(c, r, t));
      bool any = false, cert = false;
      std::vector<uint8_t> passed(n, 0);
      for (int k = 0; k < n; ++k)
        if (c->inst_on[k])
          {
            nits[k] = it + 1;
            gits[k] += its[k];
            fres[k] = r[k];
            c->stop_ls[k] = c->stop_fp64[k] = r[k];
            if (r[k] <= converge_acc)
              {
                passed[k] = 1;
                cert |= c->mixed;
              }
          }
      if (cert)
        {
          // mixed mode: the line search's double-float |R| passed; the stop test itself is
          // taken on the FP64 residual at the accepted state (run.cc:234 in FP64).  R then
          // holds the FP64 values at x, which the next assembly reuses
          CKS(upload_act(c, c->d_act, passed));
          CKS(residual_at(c, c->x, c->d_act, false, true));
          std::vector<double> r64;
          CKS(norms_d(c, c->R, c->d_act, r64));
          for (int k = 0; k < n; ++k)
            if (passed[k])
              {
                c->stop_fp64[k] = fres[k] = r64[k];
                c->res_norm[k] = r64[k];
                if (!std::isfinite(r64[k]))
                  return set_error(GLGPU_ERR_NAN, "run: non-finite FP64 residual in instance " + std::to_string(k));
                if (r64[k] > converge_acc) passed[k] = 0; // one more Newton step
              }
        }
      for (int k = 0; k < n; ++k)
        if (c->inst_on[k])
          {
            if (passed[k])
              c->inst_on[k] = 0;
            else
              any = true;
          }
      if (!any) break;
    }
  for (int k = 0; k < n; ++k)
    if (c->inst_on[k]) result = set_error(GLGPU_ERR_NOT_CONVERGED, "run: Newton iteration limit reached");
  for (int k = 0; k < n; ++k)
    if (c->handed[k])
      result = set_error(GLGPU_ERR_NOT_CONVERGED, "run: instance " + std::to_string(k) +
                                                      " handed off (its multigrid solve stalled)");
  std::fill(c->inst_on.begin(), c->inst_on.end(), 1);
  if (newton_its) std::copy(nits.begin(), nits.end(), newton_its);
  if (gmres_its) std::copy(gits.begin(), gits.end(), gmres_its);
  if (final_res) std::copy(fres.begin(), fres.end(), final_res);
  return result;
}

namespace glgpu
{
static std::atomic<bool> g_pdl{true};
bool pdl_enabled() { return g_pdl.load(std::memory_order_relaxed); }
} // namespace glgpu

extern "C" glgpu_status glgpu_set_launch_mode(int programmatic)
{
  g_pdl.store(programmatic != 0, std::memory_order_relaxed);
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_stop_norms(const glgpu_ctx *c, double *line_search_norm, double *fp64_norm)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_stop_norms: NULL context");
  if (line_search_norm) std::copy(c->stop_ls.begin(), c->stop_ls.end(), line_search_norm);
  if (fp64_norm) std::copy(c->stop_fp64.begin(), c->stop_fp64.end(), fp64_norm);
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_get_system(const glgpu_ctx *cc, int32_t *rowptr, int32_t *cols, double *vals,
                                         double *rhs)
{
  glgpu_ctx *c = const_cast<glgpu_ctx *>(cc);
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_get_system: NULL context");
  if (c->bsr_stale)
    {
      // the Hessians were not formed at this state (matrix-free step): form them, then the rows
      CKS(launch(c, KK_CELL, 1, [&] { return launch_cell(c->dm, true, c->x, c->H, nullptr, nullptr, nullptr, c->st); }));
      CKS(launch(c, KK_ROWS, 1, [&] { return launch_rows(c->dm, c->mixed, c->H, c->vals, c->st); }));
      c->bsr_stale = false;
    }
  if (rowptr) std::memcpy(rowptr, c->P.rowptr.data(), sizeof(int32_t) * c->P.rowptr.size());
  if (cols) std::memcpy(cols, c->P.cols.data(), sizeof(int32_t) * c->P.cols.size());
  const size_t nv = static_cast<size_t>(c->nnzb) * c->B * c->B;
  if (vals)
    {
      if (c->mixed && c->dm.half_vals)
        {
          std::vector<__half> tmp(nv);
          CK(cudaMemcpyAsync(tmp.data(), c->vals, sizeof(__half) * nv, cudaMemcpyDeviceToHost, c->st));
          CK(cudaStreamSynchronize(c->st));
          for (size_t i = 0; i < nv; ++i) vals[i] = static_cast<double>(__half2float(tmp[i]));
        }
      else if (c->mixed)
        {
          std::vector<float> tmp(nv);
          CK(cudaMemcpyAsync(tmp.data(), c->vals, sizeof(float) * nv, cudaMemcpyDeviceToHost, c->st));
          CK(cudaStreamSynchronize(c->st));
          for (size_t i = 0; i < nv; ++i) vals[i] = tmp[i];
        }
      else
        CK(cudaMemcpyAsync(vals, c->vals, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->st));
    }
  if (rhs) CK(cudaMemcpyAsync(rhs, c->rhs, sizeof(double) * c->N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_get_residual(const glgpu_ctx *c, double *R)
{
  if (!c || !R) return set_error(GLGPU_ERR_ARG, "glgpu_get_residual: NULL argument");
  CK(cudaMemcpyAsync(R, c->R, sizeof(double) * c->N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_get_update(const glgpu_ctx *c, double *delta)
{
  if (!c || !delta) return set_error(GLGPU_ERR_ARG, "glgpu_get_update: NULL argument");
  CK(cudaMemcpyAsync(delta, c->delta, sizeof(double) * c->N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_spmv(glgpu_ctx *c, const double *x, double *y)
{
  if (!c || !x || !y) return set_error(GLGPU_ERR_ARG, "glgpu_spmv: NULL argument");
  if (!c->has_J) return set_error(GLGPU_ERR_STATE, "glgpu_spmv: no assembled Jacobian");
  CK(cudaMemcpyAsync(c->xt, x, sizeof(double) * c->N, cudaMemcpyHostToDevice, c->st));
  CKS(axpby(c, c->xt, c->Z, nullptr, coefs(1.0, 0.0), nullptr, false, c->mixed, c->mixed));
  CKS(spmv(c, c->Z, c->Tmp, nullptr));
  CKS(axpby(c, c->Tmp, c->xt, nullptr, coefs(1.0, 0.0), nullptr, c->mixed, false, false));
  CK(cudaMemcpyAsync(y, c->xt, sizeof(double) * c->N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_timers(glgpu_ctx *c, double *phase_ms, int reset)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_timers: NULL context");
  CKS(sync(c));
  harvest(c);
  if (phase_ms)
    for (int i = 0; i < PH_N; ++i) phase_ms[i] = c->phase_ms[i];
  if (reset)
    for (int i = 0; i < PH_N; ++i) c->phase_ms[i] = 0.0;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_kernel_timing(glgpu_ctx *c, int enable, double *kernel_ms, int64_t *launches,
                                            int reset)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_kernel_timing: NULL context");
  CKS(sync(c));
  harvest(c);
  if (kernel_ms)
    for (int i = 0; i < KK_N; ++i) kernel_ms[i] = c->kms[i];
  if (launches)
    for (int i = 0; i < KK_N; ++i) launches[i] = c->klaunch[i];
  if (reset)
    for (int i = 0; i < KK_N; ++i)
      {
        c->kms[i] = 0.0;
        c->klaunch[i] = 0;
      }
  c->ktiming = enable;
  return GLGPU_OK;
}

extern "C" int64_t glgpu_launch_count(const glgpu_ctx *c)
{
  if (!c) return 0;
  int64_t n = c->launches;
  for (const glgpu_ctx *l : c->lv) n += glgpu_launch_count(l);
  return n;
}

extern "C" int64_t glgpu_device_bytes(const glgpu_ctx *c)
{
  if (!c) return 0;
  int64_t n = static_cast<int64_t>(c->dev_bytes);
  for (const glgpu_ctx *l : c->lv) n += glgpu_device_bytes(l);
  return n;
}

extern "C" glgpu_status glgpu_mem_info(size_t *free_bytes, size_t *total_bytes)
{
  if (!free_bytes || !total_bytes) return set_error(GLGPU_ERR_ARG, "glgpu_mem_info: NULL argument");
  const cudaError_t e = cudaMemGetInfo(free_bytes, total_bytes);
  if (e != cudaSuccess) return set_error(GLGPU_ERR_CUDA, std::string("cudaMemGetInfo: ") + cudaGetErrorString(e));
  return GLGPU_OK;
}

extern "C" int glgpu_mg_levels(const glgpu_ctx *c) { return c ? c->n_levels : 0; }

extern "C" int64_t glgpu_mg_fallbacks(const glgpu_ctx *c) { return c ? c->mg_fallbacks : 0; }

extern "C" glgpu_status glgpu_set_mg_handoff(glgpu_ctx *c, int on)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_set_mg_handoff: NULL context");
  c->mg_handoff = on != 0;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_set_reorthogonalization(glgpu_ctx *c, int on)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_set_reorthogonalization: NULL context");
  c->reorth = on != 0;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_mg_handed_off(const glgpu_ctx *c, uint8_t *flags)
{
  if (!c || !flags) return set_error(GLGPU_ERR_ARG, "glgpu_mg_handed_off: NULL argument");
  std::copy(c->handed.begin(), c->handed.end(), flags);
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_mg_level_info(const glgpu_ctx *c, int level, int64_t *n_nodes, int64_t *nnzb,
                                            int64_t *p_nnz)
{
  if (!c || level < 1 || level > c->n_levels) return set_error(GLGPU_ERR_ARG, "glgpu_mg_level_info: bad level");
  const glgpu_ctx *L = c->lv[level - 1];
  if (n_nodes) *n_nodes = L->nn;
  if (nnzb) *nnzb = L->nnzb;
  if (p_nnz) *p_nnz = static_cast<int64_t>(c->tr[level - 1].h_idx.size());
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_mg_level_system(const glgpu_ctx *c, int level, int32_t *rowptr, int32_t *cols,
                                              double *vals)
{
  if (!c || level < 1 || level > c->n_levels) return set_error(GLGPU_ERR_ARG, "glgpu_mg_level_system: bad level");
  return glgpu_get_system(c->lv[level - 1], rowptr, cols, vals, nullptr);
}

extern "C" glgpu_status glgpu_mg_prolongation(const glgpu_ctx *c, int level, int32_t *ptr, int32_t *idx, double *w)
{
  if (!c || level < 1 || level > c->n_levels) return set_error(GLGPU_ERR_ARG, "glgpu_mg_prolongation: bad level");
  const glgpu_ctx::Transfer &t = c->tr[level - 1];
  if (ptr) std::memcpy(ptr, t.h_ptr.data(), sizeof(int32_t) * t.h_ptr.size());
  if (idx) std::memcpy(idx, t.h_idx.data(), sizeof(int32_t) * t.h_idx.size());
  if (w) std::memcpy(w, t.h_w.data(), sizeof(double) * t.h_w.size());
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_mg_coarse_inverse(glgpu_ctx *c, int inst, int *nd, float *inv)
{
  if (!c || !nd || c->n_levels < 1 || inst < 0 || inst >= c->n_inst || !c->d_inv)
    return set_error(GLGPU_ERR_ARG, "glgpu_mg_coarse_inverse: no multigrid hierarchy or bad instance");
  const glgpu_ctx *Lc = c->lv[c->n_levels - 1];
  int64_t off = 0;
  int n = 0;
  for (int k = 0; k <= inst; ++k)
    {
      n = static_cast<int>((Lc->P.node_off[k + 1] - Lc->P.node_off[k]) * Lc->B);
      if (k < inst) off += static_cast<int64_t>(n) * n;
    }
  *nd = n;
  if (!inv) return GLGPU_OK;
  CK(cudaStreamSynchronize(c->st));
  CK(cudaMemcpy(inv, c->d_inv + off, sizeof(float) * static_cast<size_t>(n) * n, cudaMemcpyDeviceToHost));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_sync(glgpu_ctx *c)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_sync: NULL context");
  return sync(c);
}

extern "C" glgpu_status glgpu_event_start(glgpu_ctx *c)
{
  if (!c) return set_error(GLGPU_ERR_ARG, "glgpu_event_start: NULL context");
  CK(cudaEventRecord(c->ev_user0, c->st));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_event_stop(glgpu_ctx *c, double *ms)
{
  if (!c || !ms) return set_error(GLGPU_ERR_ARG, "glgpu_event_stop: NULL argument");
  CK(cudaEventRecord(c->ev_user1, c->st));
  CK(cudaEventSynchronize(c->ev_user1));
  float f = 0.f;
  CK(cudaEventElapsedTime(&f, c->ev_user0, c->ev_user1));
  *ms = f;
  return GLGPU_OK;
}
