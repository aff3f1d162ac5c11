// Host side of the geometric multigrid preconditioner: level meshes and the
// inter-level operators, built once per mesh.
//
// The reference preconditions its Krylov solve with Trilinos ML AMG
// (femgl/src/solve.cc:141-152).  Here every instance of a context that is an
// axis-aligned box with a uniform tensor grid (no hanging nodes) gets a hierarchy of
// coarser box grids with ceil(n/2) cells per axis, down to one cell per axis.  Coarse
// operators are rediscretised (the same assembly kernels on the coarse grid, at the
// state interpolated from the finer level); corrections move between levels by
// trilinear interpolation P (coarse -> fine) and its transpose (fine -> coarse).
#include <algorithm>
#include <cmath>
#include <string>

#include "glgpu_internal.h"

namespace glgpu
{
namespace
{
// node id of lattice point (i, j, k) on a box grid with n cells per axis (mesh_box order)
inline int64_t grid_node(const int *n, int64_t i, int64_t j, int64_t k)
{
  return (k * (n[1] + 1) + j) * (n[0] + 1) + i;
}
} // namespace

// A mesh is a uniform box grid when it has no hanging nodes and its node count matches
// (nx+1)(ny+1)(nz+1) for the cell counts implied by the cell size.
bool infer_box(const glgpu_mesh &m, BoxGeom &g)
{
  if (m.dim != 3 || m.n_nodes <= 0 || m.n_cells <= 0) return false;
  if (m.hang_ptr && m.hang_ptr[m.n_nodes] > 0) return false;
  for (int d = 0; d < 3; ++d)
    {
      g.lo[d] = 1e300;
      g.hi[d] = -1e300;
    }
  for (int64_t i = 0; i < m.n_nodes; ++i)
    for (int d = 0; d < 3; ++d)
      {
        g.lo[d] = std::min(g.lo[d], m.xyz[3 * i + d]);
        g.hi[d] = std::max(g.hi[d], m.xyz[3 * i + d]);
      }
  const int32_t *c = m.cells;
  for (int d = 0; d < 3; ++d)
    {
      const double h = m.xyz[3 * c[7] + d] - m.xyz[3 * c[0] + d];
      if (!(h > 0)) return false;
      g.n[d] = static_cast<int>(std::lround((g.hi[d] - g.lo[d]) / h));
      if (g.n[d] < 1) return false;
    }
  if (static_cast<int64_t>(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1) != m.n_nodes) return false;
  if (static_cast<int64_t>(g.n[0]) * g.n[1] * g.n[2] != m.n_cells) return false;
  // every node must sit on the lattice in mesh_box order
  for (int64_t i = 0; i < m.n_nodes; ++i)
    {
      int64_t ijk[3];
      for (int d = 0; d < 3; ++d)
        {
          const double t = (m.xyz[3 * i + d] - g.lo[d]) / (g.hi[d] - g.lo[d]) * g.n[d];
          ijk[d] = std::llround(t);
          if (std::fabs(t - ijk[d]) > 1e-6) return false;
        }
      if (grid_node(g.n, ijk[0], ijk[1], ijk[2]) != i) return false;
    }
  // which axis' faces carry a zero-Dirichlet mask (orbital column of that axis)
  for (int d = 0; d < 3; ++d) g.dir[d] = 0;
  if (m.dirichlet_mask)
    for (int64_t i = 0; i < m.n_nodes; ++i)
      for (int d = 0; d < 3; ++d)
        if ((m.dirichlet_mask[i] & column_mask(d)) == column_mask(d)) g.dir[d] = 1;
  return true;
}

// trilinear interpolation from box grid `src` to the given points: CSR over points
void trilinear(const BoxGeom &src, const double *pts, int64_t npts, std::vector<int32_t> &ptr,
               std::vector<int32_t> &idx, std::vector<double> &w, int64_t src_node_offset)
{
  ptr.assign(npts + 1, 0);
  idx.clear();
  w.clear();
  double h[3];
  for (int d = 0; d < 3; ++d) h[d] = (src.hi[d] - src.lo[d]) / src.n[d];
  for (int64_t p = 0; p < npts; ++p)
    {
      int64_t cell[3];
      double t[3];
      for (int d = 0; d < 3; ++d)
        {
          const double u = (pts[3 * p + d] - src.lo[d]) / h[d];
          int64_t c0 = static_cast<int64_t>(std::floor(u));
          c0 = std::min<int64_t>(std::max<int64_t>(c0, 0), src.n[d] - 1);
          cell[d] = c0;
          t[d] = std::min(1.0, std::max(0.0, u - static_cast<double>(c0)));
        }
      for (int v = 0; v < 8; ++v)
        {
          double wt = 1.0;
          for (int d = 0; d < 3; ++d) wt *= ((v >> d) & 1) ? t[d] : 1.0 - t[d];
          if (wt < 1e-14) continue;
          idx.push_back(static_cast<int32_t>(src_node_offset +
                                             grid_node(src.n, cell[0] + (v & 1), cell[1] + ((v >> 1) & 1),
                                                       cell[2] + ((v >> 2) & 1))));
          w.push_back(wt);
        }
      ptr[p + 1] = static_cast<int32_t>(idx.size());
    }
}

void transpose_csr(int64_t nrows, int64_t ncols, const std::vector<int32_t> &ptr, const std::vector<int32_t> &idx,
                   const std::vector<double> &w, std::vector<int32_t> &tptr, std::vector<int32_t> &tidx,
                   std::vector<double> &tw)
{
  tptr.assign(ncols + 1, 0);
  for (int32_t j : idx) tptr[j + 1]++;
  for (int64_t c = 0; c < ncols; ++c) tptr[c + 1] += tptr[c];
  tidx.resize(idx.size());
  tw.resize(w.size());
  std::vector<int32_t> fill(tptr.begin(), tptr.end() - 1);
  for (int64_t r = 0; r < nrows; ++r)
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k)
      {
        const int32_t c = idx[k];
        tidx[fill[c]] = static_cast<int32_t>(r);
        tw[fill[c]] = w[k];
        fill[c]++;
      }
}

// Levels below the instance meshes: level l+1 halves (rounding up) every axis of level l,
// down to one cell per axis.  All instances must be uniform boxes; returns the number of
// coarse levels (0 when multigrid does not apply).
int build_hierarchy(const glgpu_mesh *mesh, int n_inst, int max_levels, std::vector<MgLevel> &levels,
                    std::string &why)
{
  levels.clear();
  std::vector<BoxGeom> geo(n_inst);
  for (int k = 0; k < n_inst; ++k)
    if (!infer_box(mesh[k], geo[k]))
      {
        why = "instance " + std::to_string(k) + " is not a uniform box grid";
        return 0;
      }
  std::vector<BoxGeom> cur = geo;
  for (int l = 0; l < max_levels; ++l)
    {
      bool all_min = true;
      for (auto &g : cur)
        for (int d = 0; d < 3; ++d)
          if (g.n[d] > 1) all_min = false;
      if (all_min) break;
      MgLevel L;
      L.geom.resize(n_inst);
      L.meshes.resize(n_inst);
      for (int k = 0; k < n_inst; ++k)
        {
          BoxGeom c = cur[k];
          for (int d = 0; d < 3; ++d) c.n[d] = std::max(1, (cur[k].n[d] + 1) / 2);
          L.geom[k] = c;
          if (mesh_box(c.lo, c.hi, c.n, 0.0, c.dir, L.meshes[k]) != 0)
            {
              why = "coarse mesh generation failed";
              levels.clear();
              return 0;
            }
        }
      levels.push_back(std::move(L));
      cur = levels.back().geom;
    }
  return static_cast<int>(levels.size());
}

} // namespace glgpu
