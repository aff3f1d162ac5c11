// Internal declarations shared by the host and device translation units.
#pragma once

#include <cstdint>
#include <string>
#include <array>
#include <new>
#include <type_traits>
#include <utility>
#include <vector>

#include "glgpu.h"

namespace glgpu
{
// ---------------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------------
glgpu_status set_error(glgpu_status s, const std::string &msg);

// Allocator that leaves elements default-initialised (for arithmetic types: not zeroed) when a
// vector grows by resize: the multi-gigabyte multigrid term tables are written in full by a
// parallel pass, which then also takes their first-touch page faults, instead of a serial
// zero fill before it.
template <typename T> struct NoInitAlloc : std::allocator<T>
{
  template <typename U> struct rebind
  {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <typename U> NoInitAlloc(const NoInitAlloc<U> &) noexcept {}
  template <typename U> void construct(U *p) noexcept(std::is_nothrow_default_constructible<U>::value)
  {
    ::new (static_cast<void *>(p)) U;
  }
  template <typename U, typename... A> void construct(U *p, A &&...a)
  {
    ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
  }
};
template <typename T> using bulk_vector = std::vector<T, NoInitAlloc<T>>;

// ---------------------------------------------------------------------------------
// host helpers (host_util.cc)
// ---------------------------------------------------------------------------------
struct BoxMesh
{
  int nn = 0, nc = 0;
  std::vector<double> xyz;
  std::vector<int32_t> cells, hptr, hpar;
  std::vector<double> hw;
  std::vector<uint32_t> mask;
};
int matep_eval(double p, double t, bool scc, double *out);
// dir3: zero-Dirichlet (orbital column of that axis) on the x, y, z faces
// refine: per cell of the n-grid (x fastest), > 0 refines it once; nullptr refines the cells
// within `band` of a z face
int mesh_box(const double *lo, const double *hi, const int *n, double band, const int *dir3, BoxMesh &m,
             const int8_t *refine = nullptr);

// ---------------------------------------------------------------------------------
// multigrid hierarchy (mg.cc)
// ---------------------------------------------------------------------------------
struct BoxGeom
{
  double lo[3], hi[3];
  int n[3];
  int dir[3];
  int per[3]; // upper face identified with the lower one (periodic axis)
};
// tensor grid of one instance on a multigrid level: node lines per axis, Dirichlet faces,
// periodic axes
struct TensorGrid
{
  std::vector<double> x[3];
  int dir[3];
  int per[3] = {0, 0, 0};
};
// 1D interpolation of one fine node line from at most two coarse lines
struct Lin1
{
  int n;
  int c[2];
  double w[2];
};
struct MgLevel
{
  std::vector<TensorGrid> grid;                   // per instance
  std::vector<BoxMesh> meshes;                    // per instance
  std::vector<std::array<std::vector<Lin1>, 3>> map; // per instance: fine line -> coarse lines
  // per instance: 1 when the finer level is the instance's once-refined mesh and this level
  // its base grid (prolongation by interpolation at the fine node coordinates, map unused)
  std::vector<uint8_t> coord;
};
bool infer_box(const glgpu_mesh &m, BoxGeom &g);
bool infer_refined_box(const glgpu_mesh &m, BoxGeom &g);
void coord_prolongation(const glgpu_mesh &m, const TensorGrid &c, std::vector<int32_t> &ptr, std::vector<int32_t> &idx,
                        std::vector<double> &w, int64_t coarse_offset);
int mesh_tensor(const TensorGrid &g, BoxMesh &m);
void tensor_prolongation(const TensorGrid &f, const std::vector<Lin1> *map, std::vector<int32_t> &ptr,
                         std::vector<int32_t> &idx, std::vector<double> &w, int64_t coarse_offset, const int *nc);
// Transpose of a CSR matrix that is block diagonal over parts (rows row_off[k]..row_off[k+1]
// couple only to columns col_off[k]..col_off[k+1]): per part on all host threads, each
// column's entries in ascending row order.  False (outputs unspecified) when an entry lies
// outside its block.
bool transpose_csr(const std::vector<int64_t> &row_off, const std::vector<int64_t> &col_off,
                   const std::vector<int32_t> &ptr, const std::vector<int32_t> &idx, const std::vector<double> &w,
                   std::vector<int32_t> &tptr, std::vector<int32_t> &tidx, std::vector<double> &tw);
int build_hierarchy(const glgpu_mesh *mesh, int n_inst, int max_levels, std::vector<MgLevel> &levels,
                    std::string &why);
double gaussian(uint64_t seed, uint64_t index);

// Dirichlet mask of the orbital column `axis` of u and v: components 9p + 3mu + axis.
inline uint32_t column_mask(int axis)
{
  uint32_t m = 0;
  for (int part = 0; part < 2; ++part)
    for (int mu = 0; mu < 3; ++mu) m |= 1u << (9 * part + 3 * mu + axis);
  return m;
}

// ---------------------------------------------------------------------------------
// Assembly plan built on the host once per mesh (plan.cc).
//
// Rows are all nodes of all instances (global node ids).  A hanging node's row
// holds only its diagonal block.  For a regular row n, a "contribution" is a pair
// (cell e, local vertex a) whose vertex expands to n (itself with weight 1, or a
// hanging vertex whose parent is n with weight 1/2 or 1/4).  For every local vertex b
// of that cell the contribution lists where the (a,b) block lands in row n: a slot
// (position in the row) when b is a regular node, or an entry of the hanging-target
// table when b is hanging (up to 4 parent slots with weights).
// ---------------------------------------------------------------------------------
constexpr int kMaxParents = 4;

struct HangTarget
{
  int32_t count;
  int32_t slot[kMaxParents];
  double w[kMaxParents];
};

struct Plan
{
  int dim = 3, B = 18, nv = 8;
  int n_inst = 0;
  int64_t nn = 0, nc = 0, nnzb = 0;
  std::vector<int64_t> node_off, cell_off;   // per instance, size n_inst+1
  std::vector<int32_t> cells;                 // [nc][nv] global node ids
  std::vector<double> cell_h;                 // [nc][3] box edge lengths (z = 1 for 2D)
  std::vector<double> cell_x0;                // [nc][3] coordinates of local vertex 0
  std::vector<int32_t> cell_inst;             // [nc]
  std::vector<int32_t> node_inst;             // [nn]
  std::vector<uint32_t> mask;                 // [nn]
  std::vector<int32_t> hptr, hpar;            // [nn+1], global parents
  std::vector<double> hw;
  std::vector<int32_t> rowptr;                // block CSR pattern
  bulk_vector<int32_t> cols;
  std::vector<int32_t> diag;                  // [nn] index of the diagonal block
  std::vector<int32_t> rc_ptr;                // [nn+1] contributions per row
  // the per-contribution tables are written in full by the plan's parallel row pass
  bulk_vector<int32_t> rc_cell;
  bulk_vector<int32_t> rc_a;
  bulk_vector<double> rc_w;
  bulk_vector<int16_t> rc_slot;               // [ncontrib][nv]: slot, or -1 - (index into hang_tg - ht_off[row])
  std::vector<HangTarget> hang_tg;            // zero-initialised: its padding is uploaded too
  std::vector<int64_t> ht_off;                // [nn+1] first hanging target of each row
  int max_row_blocks = 0;
  // rows of the specialised 3D row kernel (full 27-block stencil, eight unit-weight cell
  // contributions, no constraint on the row) and all other rows
  std::vector<int32_t> reg_rows, gen_rows;
  // per instance: 1 when every cell has the same box edges (inst_h, [n_inst][3])
  std::vector<uint8_t> inst_uniform;
  std::vector<double> inst_h;
  // reduction segments: every segment lies inside one instance's vector range
  int seg_len = 0;
  std::vector<int64_t> seg_begin, seg_end;    // element ranges (in units of scalars)
  std::vector<int32_t> seg_inst;
  std::vector<int32_t> inst_seg_off;          // [n_inst+1]
};

// Validates the meshes and builds the plan; returns 0 or sets an error message.
glgpu_status build_plan(const glgpu_mesh *mesh, int n_inst, Plan &plan);

// Transfer between multigrid level l (the instance meshes for l = 0, plan FP) and level
// l + 1 (plan CP) of the hierarchy lv (mg.cc): the prolongation between the free spaces (pp,
// pi, pw: rows of the fine nodes, constrained fine nodes empty, constrained coarse nodes
// replaced by their parents), its transpose (rp, ri, rw), and the Galerkin term lists of
// every coarse block (g_toff over coarse blocks, g_row, fine block g_blk with weight g_w).
struct TransferTables
{
  std::vector<int32_t> pp, pi, rp, ri, g_row;
  std::vector<double> pw, rw;
  bulk_vector<int32_t> g_blk;
  bulk_vector<double> g_w;  // term weights in FP64 (fp32_weights false)
  bulk_vector<float> g_wf;  // or rounded once to FP32 (fp32_weights true; g_w stays empty)
  std::vector<int64_t> g_toff;
  // the coarse Jacobian is symmetric (a Galerkin product of the Hessian of a real functional):
  // only the blocks on or above the block diagonal (column >= row) get Galerkin terms (g_up);
  // each block below is the transpose of its mirror, g_lo = {block, mirror block} pairs
  std::vector<int32_t> g_up, g_lo;
};
glgpu_status transfer_tables(const glgpu_mesh *mesh, int n_inst, const std::vector<MgLevel> &lv, int l,
                             const Plan &FP, const Plan &CP, TransferTables &T, bool fp32_weights = false);

// Robin (AdGR) faces of the 3D cells: bit f = 2 * axis + side of robin[e] is set when face f
// of cell e is a pair-breaking boundary face (femgl/src/assemble.cc:286-348, boundary ids
// 2/3/4 carrying the zero-Dirichlet normal column).  Only cells of instances with
// active[inst] != 0 are marked.
void robin_faces(const Plan &plan, const std::vector<uint8_t> &active, std::vector<uint8_t> &robin);

// Interior face pairs of the 3D cells for the Kelly error estimator (kelly.cc).  Pair k joins
// face fa[k] (= 2 axis + side) of cell a[k] with face fb[k] of cell b[k]; the integration
// domain is cell a's face, which lies inside cell b's face: ob[k] = bit 0 / 1 set when it is
// the upper half of b's face along the first / second tangential axis, sub[k] = 1 when b's
// face is twice as large (coarse-fine interface), 0 when the faces coincide.  Faces
// identified by periodic constraints are interior pairs.  cell_ptr / cell_pair list the
// pairs each cell takes part in.
struct KellyFaces
{
  std::vector<int32_t> a, b;
  std::vector<int8_t> fa, fb, ob, sub;
  std::vector<int32_t> cell_ptr, cell_pair;
};
glgpu_status kelly_faces(const Plan &plan, KellyFaces &out);

} // namespace glgpu
