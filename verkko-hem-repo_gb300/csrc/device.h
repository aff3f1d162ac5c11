// Device-side data of one context and the launchers the context code calls.
// All launchers enqueue on the given stream and return cudaError_t of the launch.
#pragma once

#include <cstdint>
#include <utility>

#include <cuda_runtime.h>
#include <cuda_fp16.h>

namespace glgpu
{
// Programmatic dependent launch.  The solve's kernels are launched with
// cudaLaunchAttributeProgrammaticStreamSerialization, so a kernel's CTAs may be scheduled
// while the kernel before it in the stream is finishing.  Every such kernel executes
// pdl_wait() (griddepcontrol.wait: the previous grid has completed and its writes are
// visible) before it touches memory, in every CTA, so ordering stays transitive along the
// stream; pdl_trigger() then lets its own successor be scheduled.  glgpu_set_launch_mode
// turns the attribute off (plain stream order) for comparison.
bool pdl_enabled();

template <typename... KArgs, typename... Args>
inline cudaError_t pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args &&...args)
{
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

#ifdef __CUDACC__
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
#endif

constexpr int kNS3 = 171;   // unique entries of a symmetric 18x18 block
constexpr int kCoef = 9;    // {K1, K2+K3, alpha, beta1..beta5, K1/bt (0: no Robin term)}
constexpr int kSegThreads = 256;
constexpr int kSegMax = 1024;   // scalars per reduction segment (one CTA each)

// Per-cell geometry of an axis-aligned box cell: {1/hx, 1/hy, 1/hz, hx*hy*hz}.
struct __align__(32) GeoD
{
  double x, y, z, w;
};

// Mesh and plan arrays resident on the device (read-only during solves).
struct DevMesh
{
  int dim, B, nv, n_inst;
  int64_t nn, nc, nnzb;
  int max_row_blocks;
  const int32_t *cells;       // [nc][nv]
  const double *cell_h;       // [nc][3]
  const GeoD *geo_d;       // [nc] {1/hx, 1/hy, 1/hz, hx*hy*hz}
  const float4 *geo_f;        // same in FP32 (the FP32 kernels never touch the FP64 pipe)
  const float *coef_f;        // [n_inst][kCoef] FP32 copy of coef
  const float *rc_wf;         // FP32 copy of rc_w
  const int32_t *cell_inst;   // [nc]
  const int32_t *node_inst;   // [nn]
  const uint32_t *mask;       // [nn]
  const int32_t *hptr, *hpar; // hanging CSR
  const double *hw;
  const int32_t *rowptr, *cols, *diag;
  const int32_t *rc_ptr, *rc_cell, *rc_a;
  const double *rc_w;
  const int16_t *rc_slot;
  const int64_t *ht_off;
  const void *hang_tg;        // HangTarget[]
  const double *coef;         // [n_inst][kCoef]
  // segments for per-instance reductions over scalar vectors (length nn*B)
  int n_seg;
  const int64_t *seg_begin, *seg_end;
  const int32_t *seg_inst;
  const int32_t *inst_seg_off;
  const int64_t *cell_off;    // [n_inst+1]
  const int64_t *node_off_ptr; // [n_inst+1]
  // row kernel partition (3D): full interior rows and the rest
  const int32_t *reg_rows, *gen_rows;
  int64_t n_reg, n_gen;
  // per instance: the gradient (K1, K2+K3) part of a full interior row, [n_inst][27][324]
  // (zero for instances without uniform cells, whose rows are never regular)
  const double *reg_tmpl_d;
  const float *reg_tmpl_f;
  // the block values are stored in FP16 (coarse multigrid levels of a mixed context); the
  // kernels that read them widen to FP32
  int half_vals;
  // Robin (AdGR) faces: per cell the bits f = 2 axis + side of its pair-breaking faces
  // (nullptr when no instance has an active Robin term) and the cells with any
  const uint8_t *robin;
  const int32_t *robin_cells;
  int64_t n_robin;
  // some node has a constraint row (hanging node or periodic image): gathers must expand them
  int has_constraints;
  // [nn][8] offsets cell * 144 + vertex * 18 of each node's cell contributions (list order, -1
  // past the end), on meshes whose contributions all have weight 1 and number at most 8 per
  // node (no constraint rows); nullptr elsewhere
  const int32_t *rc_off8;
  // [nn][27] the block-column ids of each row (CSR order, -1 past the end) on 18x18 levels whose
  // rows have at most 27 blocks (box grids): the row kernels read them without waiting for the
  // row bounds; nullptr elsewhere
  const int32_t *cols27;
};

#ifdef __CUDACC__
// Robin weight between cell vertices a and b for component column `col` (= c % 3):
// wR sum over the cell's Robin faces f (axis != col) holding both a and b of
// int_f phi_a phi_b dS = area_f (1/9, 1/18, 1/36 for 0, 1, 2 differing tangential bits).
// ih = {1/hx, 1/hy, 1/hz}, vol = hx hy hz, so area_f = vol ih[axis].
template <typename T>
__device__ __forceinline__ T robin_weight(int bits, int a, int b, int col, T wR, T vol, T i0, T i1, T i2)
{
  T s = T(0);
#pragma unroll
  for (int f = 0; f < 6; ++f)
    {
      const int ax = f >> 1, side = f & 1;
      if (!((bits >> f) & 1) || ax == col || ((a >> ax) & 1) != side || ((b >> ax) & 1) != side) continue;
      const int diff = __popc((a ^ b) & 7);
      const T mab = diff == 0 ? T(1) / T(9) : (diff == 1 ? T(1) / T(18) : T(1) / T(36));
      s += mab * vol * (ax == 0 ? i0 : (ax == 1 ? i1 : i2));
    }
  return wR * s;
}
#endif

// ---- assembly (kernels_asm.cu) ----
// Per-cell quadrature data: H [nc][nq][NS] (type T) and/or cell residual
// r_cell [nc][nv*B] (double) and per-cell free energy (double).  fp32 with r_cell and no H
// (3D, 18 components: the mixed mode's residual) evaluates the residual in double-float
// arithmetic on the FP32 pipe; otherwise the residual is FP64.
cudaError_t launch_cell(const DevMesh &m, bool fp32, const double *x, void *H, double *r_cell, double *e_cell,
                        const uint8_t *inst_active, cudaStream_t s);
// Gradient part of a full interior row (27 blocks [27][324], slots as in the row kernel)
// for cells with edges h and coefficients K1, K2+K3.
void regular_row_stiffness(double K1, double K23, const double *h, double *out);
// Row gather of the condensed Jacobian from H (type fp32 ? float : double) into vals.
cudaError_t launch_rows(const DevMesh &m, bool fp32, const void *H, void *vals, cudaStream_t s);
// Robin face terms added into the per-cell outputs of the Robin cells (after the cell
// kernels, before the gathers): r_cell += wR M x (and e_cell += x . wR M x when e_cell)
// from the FP64 state x, or ycell += wR M z from the FP32 direction z expanded through the
// constraints and column masks like the matrix-free cell kernel does.
cudaError_t launch_robin_res(const DevMesh &m, const double *x, double *r_cell, double *e_cell, const uint8_t *act,
                             cudaStream_t s);
cudaError_t launch_robin_mf(const DevMesh &m, const float *z, float *ycell, const uint8_t *act, cudaStream_t s);

// ---- Kelly error estimator and refinement flags (kernels_est.cu) ----
// I[np] face-pair integrals of |[du/dn]|^2 and eta[nc] = sqrt(diam/24 sum of the cell's I)
cudaError_t launch_kelly(const DevMesh &m, const double *x, const int32_t *pa, const int32_t *pb, const int8_t *fa,
                         const int8_t *ob, const int8_t *sub, int64_t np, const int32_t *cptr, const int32_t *cpair,
                         double *I, float *eta, cudaStream_t s);
// hist[n_inst][256]: bits [shift, shift+8) of the estimates whose higher bits equal prefix[inst]
cudaError_t launch_radix_hist(const DevMesh &m, const float *eta, const uint32_t *prefix, int shift, uint32_t *hist,
                              cudaStream_t s);
cudaError_t launch_flags(const DevMesh &m, const float *eta, const uint32_t *thr_refine, const uint32_t *thr_coarsen,
                         int8_t *flags, cudaStream_t s);

// Condensed residual R [nn*B] from r_cell.
cudaError_t launch_res_gather(const DevMesh &m, const double *r_cell, double *R, const uint8_t *inst_active,
                              cudaStream_t s);
cudaError_t init_constants();

// ---- linear algebra (kernels_la.cu) ----
cudaError_t launch_spmv(const DevMesh &m, bool fp32, const void *vals, const void *x, void *y, const uint8_t *act,
                        cudaStream_t s, const void *b = nullptr);
// Matrix-free FP32 Jacobian at the state xs [Nn][18] (FP32 copy of the distributed Newton
// state; 3D, 18 components): the bulk Hessian is applied at each quadrature point from the
// interpolated state without forming it.
// mode 0: y = J z, 1: y = b - J z, 2: y = z + omega D^-1 (b - J z) with D^-1 [Nn][324]
// (FP16: the finest level's l1 block-Jacobi smoother).  ycell [Nc][8][18] is scratch;
// constrained rows act as the identity.
cudaError_t launch_mf(const DevMesh &m, const float *xs, const float *z, float *ycell, float *y, const float *b,
                      const __half *dinv, float omega, int mode, const uint8_t *act, cudaStream_t s,
                      int cells_per_cta = 8);
// One fused block-Jacobi sweep: y = z + omega D^-1 (b - A z); z == nullptr gives
// y = omega D^-1 b.  18x18 blocks only; y must not alias z.
cudaError_t launch_smooth(const DevMesh &m, bool fp32, const void *vals, const void *dinv, const void *b, const void *z,
                          void *y, double omega, const uint8_t *act, cudaStream_t s);
// l1: add each row's absolute off-block sum to its diagonal (l1 block-Jacobi smoother)
cudaError_t launch_bj_setup(const DevMesh &m, bool fp32, const void *vals, void *dinv, cudaStream_t s, bool l1 = false);
// the l1 smoother of a mixed context's finest level (FP32 or FP16 blocks in), inverse blocks
// stored in FP16 (computed in FP64 arithmetic like the others); 18x18 blocks
cudaError_t launch_bj_setup_half(const DevMesh &m, const void *vals, __half *dinv, cudaStream_t s);
// y = omega D^-1 b with FP16 inverse blocks (the finest level's first sweep from zero)
cudaError_t launch_smooth_zero_half(const DevMesh &m, const __half *dinv, const float *b, float *y, double omega,
                                    const uint8_t *act, cudaStream_t s);
cudaError_t launch_bj_apply(const DevMesh &m, bool fp32, const void *dinv, const void *x, void *y,
                            const uint8_t *inst_active, cudaStream_t s);
// partial[s][v] = sum over segment s of X[v][i] * y[i], v < nv (X rows strided by ld)
cudaError_t launch_seg_mdot(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, const void *y,
                            double *partial, const uint8_t *inst_active, cudaStream_t s);
// out[inst][v] = sum of partial[s][v] over the instance's segments (ld_out = stride of out per inst)
cudaError_t launch_seg_finalize(const DevMesh &m, const double *partial, int nvec, double *out, int ld_out,
                                int take_sqrt, cudaStream_t s);
// y -= sum_v coef[inst][v] X[v]   (coef ld = ldc doubles per instance)
cudaError_t launch_seg_maxpy(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, const double *coef,
                             int ldc, void *y, const uint8_t *inst_active, cudaStream_t s);
// y_seg -= sum_v coef[inst][v] X[v]; then partial2[s][v] = X[v].y (v < nvec2) and,
// when partial_norm != NULL, partial_norm[s] = y.y, from the updated y in one pass
cudaError_t launch_seg_update(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, const double *coef,
                              int ldc, void *y, int nvec2, double *partial2, double *partial_norm,
                              const uint8_t *inst_active, cudaStream_t s);
// generic per-instance vector update: y = a[inst]*x + b[inst]*y (+ c[inst]*z when z != NULL);
// a, b, c index per instance with the given strides (stride 0 = a scalar held at a[0])
struct Axpby
{
  const double *a;
  int sa;
  const double *b;
  int sb;
  const double *c;
  int sc;
  double a0, b0, c0; // used when the pointer is NULL
};
cudaError_t launch_seg_axpby(const DevMesh &m, bool x32, const void *x, bool y32, void *y, bool z32, const void *z,
                             const Axpby &k, const uint8_t *inst_active, cudaStream_t s);
// x_trial = distribute(x + a[inst] * delta) for active instances
cudaError_t launch_trial(const DevMesh &m, const double *x, const double *delta, const double *a, double *xt,
                         const uint8_t *inst_active, cudaStream_t s);
// v <- distribute(v) (hanging = weighted parents, Dirichlet = 0), double vector
cudaError_t launch_distribute(const DevMesh &m, double *v, cudaStream_t s);
// out[inst] = sum of e_cell over the instance's cells (deterministic)
cudaError_t launch_cell_sum(const DevMesh &m, const double *e_cell, double *out, cudaStream_t s);

// GMRES small dense work (per instance, one thread each)
struct GmresDev
{
  int m;                 // restart length
  double *H;             // [n_inst][(m+1)*m] column-major Hessenberg
  double *cs, *sn;       // [n_inst][m]
  double *g;             // [n_inst][m+1]
  double *y;             // [n_inst][m]
  double *hcol;          // [n_inst][m+2] column under construction (h_0..h_j, h_{j+1})
  double *hcol2;         // second CGS pass
  double *beta;          // [n_inst] norms
  double *tol;           // [n_inst] absolute tolerance
  double *res_est;       // [n_inst] current residual estimate
  int *its;              // [n_inst] columns used in this cycle
  uint8_t *active;       // [n_inst] still iterating in this cycle
  double *inv_scale;     // [n_inst] 1/h_{j+1,j} (0 on breakdown)
};
// Arnoldi step kernels with in-kernel per-instance finalisation (cnt: per-instance
// ticket counters, zero between launches)
cudaError_t launch_arnoldi_dot(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, const void *w,
                               double *partial, double *hout, int ldh, unsigned int *cnt, const uint8_t *act,
                               cudaStream_t s);
cudaError_t launch_arnoldi_update(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, void *w, int mode,
                                  int j, double *partial, const GmresDev &g, unsigned int *cnt, cudaStream_t s);
cudaError_t launch_bj_apply_scale(const DevMesh &m, bool fp32, const void *dinv, void *x, void *y,
                                  const double *scale, const uint8_t *act, cudaStream_t s);
cudaError_t launch_gmres_start(const GmresDev &g, int n_inst, const uint8_t *solve_active, cudaStream_t s);
cudaError_t launch_gmres_column(const GmresDev &g, int n_inst, int j, cudaStream_t s);
cudaError_t launch_gmres_solve_y(const GmresDev &g, int n_inst, cudaStream_t s);
// scale factors for the new basis vector from the norm (inv_scale = 1/norm or 0)
cudaError_t launch_inv(const double *in, double *out, int n, cudaStream_t s);

// ---- multigrid (kernels_mg.cu) ----
// A transfer's entries in fixed slots per row (kProlongSlots per fine node, kRestrictSlots per
// coarse node; list order, index -1 past the end): a row's slots come in one pass of 16-byte
// loads instead of its bounds and then its entries.  idx == nullptr: the CSR lists are used.
constexpr int kProlongSlots = 8, kRestrictSlots = 28;
struct TransferSlots
{
  const int32_t *idx = nullptr;
  const void *w = nullptr; // T weights
};
// zf = base + P zc, or zf += P zc when base is nullptr (constrained components keep base)
cudaError_t launch_prolong(bool fp32, int64_t nn_f, int B, const int32_t *ptr, const int32_t *idx, const void *w,
                           const void *zc, void *zf, const uint32_t *mask_f, const int32_t *hptr_f,
                           const int32_t *node_inst, const uint8_t *act, cudaStream_t s, const void *base = nullptr,
                           TransferSlots sl = {});
cudaError_t launch_restrict(bool fp32, int64_t nn_c, int B, const int32_t *ptr, const int32_t *idx, const void *w,
                            const void *rf, void *rc, const uint32_t *mask_c, const int32_t *node_inst,
                            const uint8_t *act, cudaStream_t s, TransferSlots sl = {});
// restriction fused with the coarse level's first sweep from zero (18x18 blocks):
// rc = P^T rf, z = omega D^-1 rc
cudaError_t launch_restrict_smooth(bool fp32, int64_t nn_c, const int32_t *ptr, const int32_t *idx, const void *w,
                                   const void *rf, void *rc, const uint32_t *mask_c, const int32_t *node_inst,
                                   const uint8_t *act, const void *dinv, double omega, void *z, cudaStream_t s,
                                   TransferSlots sl = {});
// Galerkin product J_c = P^T J_f P on the coarse block pattern, one warp per coarse
// block: block cb = up[u] (row g_row[cb], column cols_c[cb] >= the row) is the sum over its
// term list [g_toff[cb], g_toff[cb+1]) of g_w * (fine block g_blk).  Zero-Dirichlet rows and
// columns and the constrained nodes (hptr_c) of the coarse level become identity rows /
// zero columns.  Then each block below the diagonal, lo[2 i], is set to the transpose of
// its mirror lo[2 i + 1] (J_c is symmetric like J_f).
// half_in / half_out: the fine / coarse blocks are stored in FP16 (mixed mode, summed in FP32).
cudaError_t launch_galerkin(bool fp32, int64_t n_up, const int32_t *up, int64_t n_lo, const int32_t *lo,
                            const int32_t *g_row, const int32_t *cols_c, const uint32_t *mask_c, const int32_t *hptr_c,
                            void *vals_c, const int64_t *g_toff, const int32_t *g_blk, const void *g_w,
                            const void *vals_f, const int32_t *node_inst_c, const uint8_t *act, cudaStream_t s,
                            bool half_in = false, bool half_out = false);
// The small coarse levels of a V-cycle fused into one cooperative launch (levels whose
// block values are FP32/FP64, 18x18 blocks): the recursion below the first such level
// (pre-sweeps beyond the one that came with the restriction, residual, restriction fused
// with the next level's first sweep, the coarsest dense solve, prolongation, post-sweeps)
// runs phase by phase over all levels and instances, separated by grid-wide barriers.
template <typename T> struct SmallLevel
{
  DevMesh m;                // the level's plan (rowptr, cols, mask, hptr, node_inst, nn)
  const T *vals, *dinv;     // block values and the l1 block-Jacobi inverse blocks
  T *r, *z, *t, *t2;        // right-hand side, iterate, residual, ping-pong buffer
  const int32_t *r_ptr, *r_idx, *p_ptr, *p_idx; // restriction to / prolongation from the next level
  const T *r_w, *p_w;
};
template <typename T> struct SmallCycle
{
  int n_small;              // smoothing levels in the fused range; levels[n_small] is the coarsest
  int pre, post;            // sweeps before / after the coarse correction
  T omega;
  int max_nd;               // coarsest dense solve
  const int64_t *dense_off;
  const float *inv;
  unsigned int *bar;        // [2]: arrival count, generation (zero at allocation)
  int *err;                 // set when a grid barrier gave up waiting
};
// levels: device array of SmallLevel<T> [n_small + 1]; grid: cooperative, all CTAs resident
cudaError_t launch_vcycle_small(bool fp32, const void *levels, const void *cycle, int grid, const uint8_t *act,
                                cudaStream_t s);
// CTAs per SM the fused small-level V-cycle is launched with (the occupancy limit, at most 4)
int vcycle_small_blocks_per_sm(bool fp32);

// The tail of a V-cycle (the few smallest levels and the dense coarsest solve) in one launch
// of one thread-block cluster per instance: the CTAs of a cluster split each phase's rows
// and meet at the cluster's hardware barrier between phases.  It starts from the parent
// level's residual (the finest level outside the tail) and ends with the parent's coarse
// correction out = cur + P e.  levels: device array of SmallLevel<T> [n_tail + 2]: [0] the
// parent (its plan and the transfers to [1]), [1 .. n_tail] the smoothing levels, [n_tail
// + 1] the dense level.
template <typename T> struct TailCycle
{
  int n_tail;               // smoothing levels in the tail (>= 1)
  int pre, post;
  T omega;
  const int64_t *dense_off;
  const float *inv;
};
// cluster size (CTAs per instance) the tail can be launched with for n_inst instances on
// this device (16, 8, 4, 2 or 1; 0: not available); also sets the kernel's attributes
int vcycle_tail_cluster(bool fp32, int n_inst);
cudaError_t launch_vcycle_tail(bool fp32, const void *levels, const void *cycle, int n_inst, int cluster,
                               const void *p_res, const void *p_cur, void *p_out, const uint8_t *act, cudaStream_t s);
cudaError_t launch_dense_setup(const DevMesh &m, bool fp32, const void *vals, const int64_t *dense_off, int max_nd,
                               float *inv, int *singular, float shift, cudaStream_t s);
cudaError_t launch_dense_apply(const DevMesh &m, bool fp32, int max_nd, const int64_t *dense_off, const float *inv,
                               const void *r, void *z, const uint8_t *act, cudaStream_t s);

} // namespace glgpu
