// Host side of the geometric multigrid preconditioner: level grids, inter-level transfer
// operators and the tables of the Galerkin products, built once per mesh.
//
// The reference preconditions its Krylov solve with Trilinos ML AMG
// (femgl/src/solve.cc:141-152).  Here every instance of a context that is an axis-aligned
// box with a tensor grid (periodic axes allowed) gets a hierarchy of nested coarser tensor
// grids: a coarsened axis keeps every other node line and the last one.  Prolongation P
// is the tensor product of 1D linear interpolation along the axes, restriction is P^T,
// and the coarse Jacobians are the Galerkin products P^T J P (formed on the GPU after each
// fine assembly), so every coarse operator is consistent with the fine Jacobian.  An axis
// whose spacing is more than twice the smallest one is left alone until the others catch
// up (semi-coarsening), so anisotropic slabs become isotropic before full coarsening.
// A box grid whose flagged cells were refined once (hanging nodes on the coarse-fine
// faces, as the reference's refine_grid produces them: femgl/src/refine.cc:131-176) has the
// unrefined grid as its first coarse level: its Q1 space contains the base grid's, and P
// interpolates the base grid's Q1 field at the fine nodes' coordinates.
#include <algorithm>
#include <cmath>
#include <string>

#include "glgpu_internal.h"

namespace glgpu
{
namespace
{
// node id of lattice point (i, j, k) on a tensor grid with n cells per axis (mesh_box order)
inline int64_t grid_node(const int *n, int64_t i, int64_t j, int64_t k)
{
  return (k * (n[1] + 1) + j) * (n[0] + 1) + i;
}

// Coarse lines of one axis and the interpolation of every fine line from them.
void line_map(const std::vector<double> &xf, bool coarsen, std::vector<double> &xc, std::vector<Lin1> &map)
{
  const int nf = static_cast<int>(xf.size()) - 1;
  xc.clear();
  map.assign(nf + 1, Lin1{});
  if (!coarsen)
    {
      xc = xf;
      for (int i = 0; i <= nf; ++i) map[i] = Lin1{1, {i, 0}, {1.0, 0.0}};
      return;
    }
  for (int i = 0; i <= nf; i += 2) xc.push_back(xf[i]);
  if (nf % 2) xc.push_back(xf[nf]);
  const int nc = static_cast<int>(xc.size()) - 1;
  for (int i = 0; i <= nf; ++i)
    {
      if (i % 2 == 0)
        map[i] = Lin1{1, {i / 2, 0}, {1.0, 0.0}};
      else if (i == nf)
        map[i] = Lin1{1, {nc, 0}, {1.0, 0.0}};
      else
        {
          const int a = (i - 1) / 2, b = a + 1;
          const double t = (xf[i] - xc[a]) / (xc[b] - xc[a]);
          map[i] = Lin1{2, {a, b}, {1.0 - t, t}};
        }
    }
}
} // namespace

// A mesh is a uniform box grid when its node count matches (nx+1)(ny+1)(nz+1) for the
// cell counts implied by the cell size and its only constraints are periodic
// identifications: on a periodic axis every node of the upper face has exactly one parent,
// weight 1, its image with every periodic coordinate at the lower face.
bool infer_box(const glgpu_mesh &m, BoxGeom &g)
{
  if (m.dim != 3 || m.n_nodes <= 0 || m.n_cells <= 0) return false;
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
  // periodic axes: every node of the upper face constrained
  auto constrained = [&](int64_t i) { return m.hang_ptr && m.hang_ptr[i + 1] > m.hang_ptr[i]; };
  for (int d = 0; d < 3; ++d) g.per[d] = 0;
  if (m.hang_ptr && m.hang_ptr[m.n_nodes] > 0)
    for (int d = 0; d < 2; ++d)
      {
        bool all = true;
        for (int k = 0; k <= g.n[2] && all; ++k)
          for (int j = 0; j <= g.n[1] && all; ++j)
            for (int i = 0; i <= g.n[0] && all; ++i)
              {
                const int64_t c3[3] = {i, j, k};
                if (c3[d] == g.n[d] && !constrained(grid_node(g.n, i, j, k))) all = false;
              }
        g.per[d] = all ? 1 : 0;
      }
  if (m.hang_ptr)
    for (int64_t i = 0; i < m.n_nodes; ++i)
      {
        if (!constrained(i)) continue;
        const int64_t ii = i % (g.n[0] + 1), jj = (i / (g.n[0] + 1)) % (g.n[1] + 1), kk = i / ((g.n[0] + 1) * (g.n[1] + 1));
        int64_t c3[3] = {ii, jj, kk};
        bool upper = false;
        for (int d = 0; d < 2; ++d)
          if (g.per[d] && c3[d] == g.n[d])
            {
              c3[d] = 0;
              upper = true;
            }
        const int32_t h0 = m.hang_ptr[i];
        if (!upper || m.hang_ptr[i + 1] - h0 != 1 || m.hang_weight[h0] != 1.0 ||
            m.hang_parent[h0] != grid_node(g.n, c3[0], c3[1], c3[2]))
          return false;
      }
  // which axis' faces carry a zero-Dirichlet mask (orbital column of that axis)
  for (int d = 0; d < 3; ++d) g.dir[d] = 0;
  if (m.dirichlet_mask)
    for (int64_t i = 0; i < m.n_nodes; ++i)
      for (int d = 0; d < 3; ++d)
        if ((m.dirichlet_mask[i] & column_mask(d)) == column_mask(d)) g.dir[d] = 1;
  for (int d = 0; d < 3; ++d)
    if (g.dir[d] && g.per[d]) return false;
  return true;
}

// A mesh is a once-refined box grid when its cells fill its bounding box, every cell is an
// axis-aligned box whose edges are those of the base grid (the largest cell's) on all three
// axes or half of them on all three axes, the base-size cells start on the base lattice,
// every node lies on the half lattice,
// and every constraint row is a hanging-node row or a periodic image (one parent, weight 1,
// displaced by the box extent along the periodic axes).  g receives the base grid.
bool infer_refined_box(const glgpu_mesh &m, BoxGeom &g)
{
  if (m.dim != 3 || m.n_nodes <= 0 || m.n_cells <= 0 || !m.xyz || !m.cells) return false;
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
  double H[3] = {0.0, 0.0, 0.0};
  for (int64_t e = 0; e < m.n_cells; ++e)
    for (int d = 0; d < 3; ++d)
      {
        const int32_t *c = m.cells + 8 * e;
        if (c[0] < 0 || c[0] >= m.n_nodes || c[7] < 0 || c[7] >= m.n_nodes) return false;
        H[d] = std::max(H[d], m.xyz[3 * c[7] + d] - m.xyz[3 * c[0] + d]);
      }
  for (int d = 0; d < 3; ++d)
    {
      const double ext = g.hi[d] - g.lo[d];
      if (!(H[d] > 0) || !(ext > 0)) return false;
      g.n[d] = static_cast<int>(std::lround(ext / H[d]));
      if (g.n[d] < 1 || std::fabs(g.n[d] * H[d] - ext) > 1e-9 * ext) return false;
    }
  // position on the half lattice of the base grid
  auto half = [&](int d, double x, int64_t &r) {
    const double u = 2.0 * (x - g.lo[d]) / (g.hi[d] - g.lo[d]) * g.n[d];
    r = std::llround(u);
    return std::fabs(u - static_cast<double>(r)) <= 1e-6;
  };
  for (int64_t i = 0; i < m.n_nodes; ++i)
    for (int d = 0; d < 3; ++d)
      {
        int64_t r;
        if (!half(d, m.xyz[3 * i + d], r)) return false;
      }
  // the cells must fill the bounding box (an L-shaped lattice domain would leave base-grid
  // nodes outside the mesh, with empty rows in the coarse operator)
  {
    double vol = 0.0;
    for (int64_t e = 0; e < m.n_cells; ++e)
      {
        const int32_t *c = m.cells + 8 * e;
        double v = 1.0;
        for (int d = 0; d < 3; ++d) v *= m.xyz[3 * c[7] + d] - m.xyz[3 * c[0] + d];
        vol += v;
      }
    const double box = (g.hi[0] - g.lo[0]) * (g.hi[1] - g.lo[1]) * (g.hi[2] - g.lo[2]);
    if (std::fabs(vol - box) > 1e-9 * box) return false;
  }
  for (int64_t e = 0; e < m.n_cells; ++e)
    {
      const int32_t *c = m.cells + 8 * e;
      int kind = -1; // 0 base size, 1 half size
      for (int d = 0; d < 3; ++d)
        {
          const double h = m.xyz[3 * c[7] + d] - m.xyz[3 * c[0] + d];
          const int k = (std::fabs(h - H[d]) <= 1e-6 * H[d]) ? 0 : (std::fabs(2.0 * h - H[d]) <= 1e-6 * H[d]) ? 1 : -1;
          if (k < 0 || (kind >= 0 && k != kind)) return false;
          kind = k;
          int64_t r;
          half(d, m.xyz[3 * c[0] + d], r);
          if (kind == 0 && (r & 1)) return false;
        }
    }
  // constraint rows: hanging nodes (at least two parents) or periodic images
  for (int d = 0; d < 3; ++d) g.per[d] = 0;
  if (m.hang_ptr)
    for (int64_t i = 0; i < m.n_nodes; ++i)
      {
        const int32_t h0 = m.hang_ptr[i], h1 = m.hang_ptr[i + 1];
        if (h1 - h0 != 1) continue;
        const int64_t p = m.hang_parent[h0];
        if (m.hang_weight[h0] != 1.0 || p < 0 || p >= m.n_nodes) return false;
        bool moved = false;
        for (int d = 0; d < 3; ++d)
          {
            const double dx = m.xyz[3 * i + d] - m.xyz[3 * p + d], ext = g.hi[d] - g.lo[d];
            if (std::fabs(dx) <= 1e-6 * H[d]) continue;
            if (std::fabs(dx - ext) > 1e-6 * H[d]) return false;
            g.per[d] = 1;
            moved = true;
          }
        if (!moved) return false;
      }
  for (int d = 0; d < 3; ++d) g.dir[d] = 0;
  if (m.dirichlet_mask)
    for (int64_t i = 0; i < m.n_nodes; ++i)
      for (int d = 0; d < 3; ++d)
        if ((m.dirichlet_mask[i] & column_mask(d)) == column_mask(d)) g.dir[d] = 1;
  for (int d = 0; d < 3; ++d)
    if (g.dir[d] && g.per[d]) return false;
  return true;
}

// Interpolation rows of the Q1 field of tensor grid c (nodes numbered as mesh_tensor numbers
// them, plus coarse_offset) at the coordinates of every node of m: the tensor product of the
// 1D linear interpolation between the two node lines around each coordinate.
void coord_prolongation(const glgpu_mesh &m, const TensorGrid &c, std::vector<int32_t> &ptr, std::vector<int32_t> &idx,
                        std::vector<double> &w, int64_t coarse_offset)
{
  int nc[3];
  for (int d = 0; d < 3; ++d) nc[d] = static_cast<int>(c.x[d].size()) - 1;
  ptr.assign(1, 0);
  idx.clear();
  w.clear();
  for (int64_t i = 0; i < m.n_nodes; ++i)
    {
      Lin1 a[3];
      for (int d = 0; d < 3; ++d)
        {
          const std::vector<double> &x = c.x[d];
          const double v = m.xyz[3 * i + d], tol = 1e-9 * (x.back() - x.front());
          int j = static_cast<int>(std::upper_bound(x.begin(), x.end(), v + tol) - x.begin()) - 1;
          j = std::max(0, std::min(j, nc[d]));
          if (j == nc[d] || std::fabs(v - x[j]) <= tol)
            a[d] = Lin1{1, {j, 0}, {1.0, 0.0}};
          else if (std::fabs(x[j + 1] - v) <= tol)
            a[d] = Lin1{1, {j + 1, 0}, {1.0, 0.0}};
          else
            {
              const double t = (v - x[j]) / (x[j + 1] - x[j]);
              a[d] = Lin1{2, {j, j + 1}, {1.0 - t, t}};
            }
        }
      for (int r = 0; r < a[2].n; ++r)
        for (int q = 0; q < a[1].n; ++q)
          for (int p = 0; p < a[0].n; ++p)
            {
              idx.push_back(static_cast<int32_t>(coarse_offset + grid_node(nc, a[0].c[p], a[1].c[q], a[2].c[r])));
              w.push_back(a[0].w[p] * a[1].w[q] * a[2].w[r]);
            }
      ptr.push_back(static_cast<int32_t>(idx.size()));
    }
}

// Hexahedral mesh of a tensor grid: nodes in (k, j, i) lexicographic order, cells in
// deal.II vertex order, zero-Dirichlet masks on the faces of the axes flagged in dir, and
// on periodic axes the upper face's nodes constrained to their images (weight 1).
int mesh_tensor(const TensorGrid &g, BoxMesh &m)
{
  int n[3];
  for (int d = 0; d < 3; ++d)
    {
      n[d] = static_cast<int>(g.x[d].size()) - 1;
      if (n[d] < 1) return -1;
    }
  const int64_t nn = static_cast<int64_t>(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
  const int64_t nc = static_cast<int64_t>(n[0]) * n[1] * n[2];
  if (nn > INT32_MAX / 32 || nc > INT32_MAX / 8) return -1;
  m.nn = static_cast<int>(nn);
  m.nc = static_cast<int>(nc);
  m.xyz.resize(nn * 3);
  m.mask.assign(nn, 0u);
  for (int k = 0; k <= n[2]; ++k)
    for (int j = 0; j <= n[1]; ++j)
      for (int i = 0; i <= n[0]; ++i)
        {
          const int64_t id = grid_node(n, i, j, k);
          m.xyz[3 * id + 0] = g.x[0][i];
          m.xyz[3 * id + 1] = g.x[1][j];
          m.xyz[3 * id + 2] = g.x[2][k];
          const int c3[3] = {i, j, k};
          bool slave = false;
          for (int d = 0; d < 3; ++d) slave = slave || (g.per[d] && c3[d] == n[d]);
          if (slave) continue; // constrained nodes carry no mask
          for (int d = 0; d < 3; ++d)
            if (g.dir[d] && (c3[d] == 0 || c3[d] == n[d])) m.mask[id] |= column_mask(d);
        }
  m.cells.resize(nc * 8);
  int64_t e = 0;
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i, ++e)
        for (int v = 0; v < 8; ++v)
          m.cells[e * 8 + v] = static_cast<int32_t>(grid_node(n, i + (v & 1), j + ((v >> 1) & 1), k + ((v >> 2) & 1)));
  m.hptr.assign(nn + 1, 0);
  m.hpar.clear();
  m.hw.clear();
  for (int k = 0; k <= n[2]; ++k)
    for (int j = 0; j <= n[1]; ++j)
      for (int i = 0; i <= n[0]; ++i)
        {
          int c3[3] = {i, j, k};
          bool slave = false;
          for (int d = 0; d < 3; ++d)
            if (g.per[d] && c3[d] == n[d])
              {
                c3[d] = 0;
                slave = true;
              }
          const int64_t id = grid_node(n, i, j, k);
          if (slave)
            {
              m.hpar.push_back(static_cast<int32_t>(grid_node(n, c3[0], c3[1], c3[2])));
              m.hw.push_back(1.0);
            }
          m.hptr[id + 1] = static_cast<int32_t>(m.hpar.size());
        }
  return 0;
}

bool transpose_csr(const std::vector<int64_t> &row_off, const std::vector<int64_t> &col_off,
                   const std::vector<int32_t> &ptr, const std::vector<int32_t> &idx, const std::vector<double> &w,
                   std::vector<int32_t> &tptr, std::vector<int32_t> &tidx, std::vector<double> &tw)
{
  const int parts = static_cast<int>(row_off.size()) - 1;
  const int64_t ncols = col_off[parts];
  tptr.assign(ncols + 1, 0);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
  for (int k = 0; k < parts; ++k)
    for (int64_t r = row_off[k]; r < row_off[k + 1]; ++r)
      for (int32_t q = ptr[r]; q < ptr[r + 1]; ++q)
        {
          if (idx[q] < col_off[k] || idx[q] >= col_off[k + 1])
            bad = 1; // an entry outside the block's columns
          else
            tptr[idx[q] + 1]++;
        }
  if (bad) return false;
  for (int64_t c = 0; c < ncols; ++c) tptr[c + 1] += tptr[c];
  tidx.resize(idx.size());
  tw.resize(w.size());
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < parts; ++k)
    {
      const int64_t c0 = col_off[k];
      std::vector<int32_t> fill(tptr.begin() + c0, tptr.begin() + col_off[k + 1]);
      for (int64_t r = row_off[k]; r < row_off[k + 1]; ++r)
        for (int32_t q = ptr[r]; q < ptr[r + 1]; ++q)
          {
            const int64_t c = idx[q] - c0;
            tidx[fill[c]] = static_cast<int32_t>(r);
            tw[fill[c]] = w[q];
            fill[c]++;
          }
    }
  return true;
}

// Prolongation of one instance from level grid `c` to the next finer grid `f` (local node
// ids): the tensor product of the per-axis maps.
void tensor_prolongation(const TensorGrid &f, const std::vector<Lin1> *map, std::vector<int32_t> &ptr,
                         std::vector<int32_t> &idx, std::vector<double> &w, int64_t coarse_offset, const int *nc)
{
  int nf[3];
  for (int d = 0; d < 3; ++d) nf[d] = static_cast<int>(f.x[d].size()) - 1;
  ptr.assign(1, 0);
  idx.clear();
  w.clear();
  for (int k = 0; k <= nf[2]; ++k)
    for (int j = 0; j <= nf[1]; ++j)
      for (int i = 0; i <= nf[0]; ++i)
        {
          const Lin1 &a = map[0][i], &b = map[1][j], &cz = map[2][k];
          for (int r = 0; r < cz.n; ++r)
            for (int q = 0; q < b.n; ++q)
              for (int p = 0; p < a.n; ++p)
                {
                  idx.push_back(static_cast<int32_t>(coarse_offset + grid_node(nc, a.c[p], b.c[q], cz.c[r])));
                  w.push_back(a.w[p] * b.w[q] * cz.w[r]);
                }
          ptr.push_back(static_cast<int32_t>(idx.size()));
        }
}

// Levels below the instance meshes, down to one cell per axis.  All instances must be
// tensor box grids or once-refined box grids (whose first coarse level is their base grid);
// returns the number of coarse levels (0 when multigrid does not apply).
int build_hierarchy(const glgpu_mesh *mesh, int n_inst, int max_levels, std::vector<MgLevel> &levels,
                    std::string &why)
{
  levels.clear();
  std::vector<TensorGrid> cur(n_inst);
  std::vector<uint8_t> refined(n_inst, 0);
  bool any_refined = false;
  for (int k = 0; k < n_inst; ++k)
    {
      BoxGeom g;
      if (!infer_box(mesh[k], g))
        {
          if (!infer_refined_box(mesh[k], g))
            {
              why = "instance " + std::to_string(k) + " is neither a box grid nor a once-refined box grid";
              return 0;
            }
          refined[k] = 1;
          any_refined = true;
        }
      for (int d = 0; d < 3; ++d)
        {
          cur[k].x[d].resize(g.n[d] + 1);
          for (int i = 0; i <= g.n[d]; ++i)
            cur[k].x[d][i] = (i == g.n[d]) ? g.hi[d] : g.lo[d] + (g.hi[d] - g.lo[d]) * i / g.n[d];
          cur[k].dir[d] = g.dir[d];
          cur[k].per[d] = g.per[d];
        }
    }
  for (int l = 0; l < max_levels; ++l)
    {
      bool all_min = true;
      for (auto &g : cur)
        for (int d = 0; d < 3; ++d)
          if (g.x[d].size() > 2) all_min = false;
      if (all_min && !(l == 0 && any_refined)) break;
      MgLevel L;
      L.grid.resize(n_inst);
      L.meshes.resize(n_inst);
      L.map.resize(n_inst);
      L.coord.assign(n_inst, 0);
      for (int k = 0; k < n_inst; ++k)
        {
          if (l == 0 && refined[k])
            {
              // the base grid itself, reached by interpolation at the fine coordinates
              L.grid[k] = cur[k];
              L.coord[k] = 1;
              if (mesh_tensor(L.grid[k], L.meshes[k]) != 0)
                {
                  why = "coarse mesh generation failed";
                  levels.clear();
                  return 0;
                }
              continue;
            }
          const TensorGrid &f = cur[k];
          double h[3], hmin = 1e300;
          for (int d = 0; d < 3; ++d)
            {
              h[d] = f.x[d].size() > 2 ? f.x[d][1] - f.x[d][0] : 1e300;
              hmin = std::min(hmin, h[d]);
            }
          TensorGrid c;
          for (int d = 0; d < 3; ++d)
            {
              const bool coarsen = f.x[d].size() > 2 && h[d] < 2.0 * hmin;
              line_map(f.x[d], coarsen, c.x[d], L.map[k][d]);
              c.dir[d] = f.dir[d];
              c.per[d] = f.per[d];
            }
          L.grid[k] = c;
          if (mesh_tensor(c, L.meshes[k]) != 0)
            {
              why = "coarse mesh generation failed";
              levels.clear();
              return 0;
            }
        }
      levels.push_back(std::move(L));
      cur = levels.back().grid;
    }
  return static_cast<int>(levels.size());
}

glgpu_status transfer_tables(const glgpu_mesh *mesh, int n_inst, const std::vector<MgLevel> &lv, int l,
                             const Plan &FP, const Plan &CP, TransferTables &T, bool fp32_weights)
{
  std::vector<int32_t> &pp = T.pp, &pi = T.pi;
  std::vector<double> &pw = T.pw;
  // prolongation rows per instance on all host threads, then concatenated in instance order;
  // err[k]: 1 = not a box grid, 2 = level grid and mesh disagree (the first failing instance
  // is reported, as a serial loop would)
  std::vector<std::vector<int32_t>> ipp(n_inst), ipi(n_inst);
  std::vector<std::vector<double>> ipw(n_inst);
  std::vector<int> err(n_inst, 0);
#pragma omp parallel
  {
    std::vector<std::pair<int32_t, double>> row; // one fine row's entries, reused
#pragma omp for schedule(dynamic, 1)
    for (int k = 0; k < n_inst; ++k)
      {
        std::vector<int32_t> a, b;
        std::vector<double> w;
        if (l == 0 && !lv[0].coord.empty() && lv[0].coord[k])
          coord_prolongation(mesh[k], lv[0].grid[k], a, b, w, CP.node_off[k]);
        else
          {
            TensorGrid fg;
            if (l == 0)
              {
                BoxGeom g;
                if (!infer_box(mesh[k], g))
                  {
                    err[k] = 1;
                    continue;
                  }
                for (int d = 0; d < 3; ++d) fg.x[d].resize(g.n[d] + 1);
              }
            else
              fg = lv[l - 1].grid[k];
            int nc[3];
            for (int d = 0; d < 3; ++d) nc[d] = static_cast<int>(lv[l].grid[k].x[d].size()) - 1;
            tensor_prolongation(fg, lv[l].map[k].data(), a, b, w, CP.node_off[k], nc);
          }
        if (static_cast<int64_t>(a.size()) - 1 != FP.node_off[k + 1] - FP.node_off[k])
          {
            err[k] = 2;
            continue;
          }
        // prolongation between the free spaces: constrained fine nodes (hanging nodes,
        // periodic images) get no row, constrained coarse nodes are replaced by their parents
        std::vector<int32_t> &lpp = ipp[k], &lpi = ipi[k];
        std::vector<double> &lpw = ipw[k];
        lpp.assign(1, 0);
        const int64_t f0 = FP.node_off[k];
        for (size_t i = 0; i + 1 < a.size(); ++i)
          {
            const int64_t fi = f0 + static_cast<int64_t>(i);
            row.clear();
            if (FP.hptr[fi + 1] == FP.hptr[fi])
              for (int32_t q = a[i]; q < a[i + 1]; ++q)
                {
                  const int32_t j = b[q];
                  if (CP.hptr[j + 1] == CP.hptr[j])
                    row.push_back({j, w[q]});
                  else
                    for (int32_t h = CP.hptr[j]; h < CP.hptr[j + 1]; ++h) row.push_back({CP.hpar[h], w[q] * CP.hw[h]});
                }
            std::sort(row.begin(), row.end());
            size_t nr = 0;
            for (size_t q = 0; q < row.size(); ++q)
              if (nr > 0 && row[nr - 1].first == row[q].first)
                row[nr - 1].second += row[q].second;
              else
                row[nr++] = row[q];
            for (size_t q = 0; q < nr; ++q)
              {
                lpi.push_back(row[q].first);
                lpw.push_back(row[q].second);
              }
            lpp.push_back(static_cast<int32_t>(lpi.size()));
          }
      }
  }
  for (int k = 0; k < n_inst; ++k)
    {
      if (err[k] == 1) return set_error(GLGPU_ERR_ARG, "multigrid: instance is not a box grid");
      if (err[k] == 2) return set_error(GLGPU_ERR_ARG, "multigrid: level grid does not match the mesh");
    }
  {
    size_t total = 0, rows = 0;
    for (int k = 0; k < n_inst; ++k)
      {
        total += ipi[k].size();
        rows += ipp[k].size() - 1;
      }
    if (total >= (size_t(1) << 31)) return set_error(GLGPU_ERR_ARG, "multigrid: prolongation too large");
    pp.assign(1, 0);
    pp.reserve(rows + 1);
    pi.clear();
    pw.clear();
    pi.reserve(total);
    pw.reserve(total);
    for (int k = 0; k < n_inst; ++k)
      {
        const int32_t base = static_cast<int32_t>(pi.size());
        for (size_t r = 1; r < ipp[k].size(); ++r) pp.push_back(base + ipp[k][r]);
        pi.insert(pi.end(), ipi[k].begin(), ipi[k].end());
        pw.insert(pw.end(), ipw[k].begin(), ipw[k].end());
        std::vector<int32_t>().swap(ipi[k]);
        std::vector<double>().swap(ipw[k]);
      }
  }
  std::vector<int32_t> &rp = T.rp, &ri = T.ri;
  std::vector<double> &rw = T.rw;
  if (!transpose_csr(FP.node_off, CP.node_off, pp, pi, pw, rp, ri, rw))
    return set_error(GLGPU_ERR_ARG, "multigrid: prolongation couples instances");
  // Galerkin terms, grouped by coarse block: every (restriction entry i of row I, fine block
  // (i, j), prolongation entry J of j) adds w(i, I) w(j, J) J_f(i, j) to block (I, J); within a
  // block the terms follow (restriction entry, fine block, prolongation entry) order, so fine
  // blocks come in increasing order.  Only blocks with J >= I get terms: the blocks below
  // the diagonal are the transposes of their mirrors.  Pass 0 counts the terms of every
  // block, pass 1 writes them at their offsets; both run over the coarse rows on all host
  // threads (a row's blocks belong to one thread), and the tables do not depend on the
  // thread count.
  std::vector<int64_t> &gt = T.g_toff;
  std::vector<int32_t> &grow = T.g_row;
  bulk_vector<int32_t> &gb = T.g_blk;
  bulk_vector<double> &gw = T.g_w;
  bulk_vector<float> &gwf = T.g_wf;
  gt.assign(static_cast<size_t>(CP.nnzb) + 1, 0);
  grow.assign(static_cast<size_t>(CP.nnzb), 0);
  const int64_t ncr = CP.nn;
  for (int pass = 0; pass < 2; ++pass)
    {
      if (pass == 1)
        {
          for (int64_t b = 0; b < CP.nnzb; ++b) gt[b + 1] += gt[b];
          // every entry is written below (pass 1 visits exactly the terms pass 0 counted)
          gb.clear();
          gw.clear();
          gwf.clear();
          gb.resize(static_cast<size_t>(gt[CP.nnzb]));
          if (fp32_weights)
            gwf.resize(static_cast<size_t>(gt[CP.nnzb]));
          else
            gw.resize(static_cast<size_t>(gt[CP.nnzb]));
        }
      int outside = 0;
#pragma omp parallel reduction(| : outside)
      {
        std::vector<int32_t> slot_of(static_cast<size_t>(ncr), -1); // column -> slot of the current row
        std::vector<int64_t> pos(static_cast<size_t>(CP.max_row_blocks));
#pragma omp for schedule(dynamic, 64)
        for (int64_t I = 0; I < ncr; ++I)
          {
            const int32_t b0 = CP.rowptr[I], ns = CP.rowptr[I + 1] - b0;
            const int32_t *c0 = CP.cols.data() + b0;
            for (int s = 0; s < ns; ++s)
              {
                slot_of[c0[s]] = s;
                if (pass == 1) pos[s] = gt[b0 + s];
              }
            for (int32_t k = rp[I]; k < rp[I + 1]; ++k)
              {
                const int32_t i = ri[k];
                for (int32_t b = FP.rowptr[i]; b < FP.rowptr[i + 1]; ++b)
                  {
                    const int32_t j = FP.cols[b];
                    for (int32_t q = pp[j]; q < pp[j + 1]; ++q)
                      {
                        const int32_t sl = slot_of[pi[q]];
                        if (sl < 0)
                          {
                            outside = 1;
                            continue;
                          }
                        if (c0[sl] < I) continue; // below the diagonal: a mirror
                        if (pass == 0)
                          ++gt[b0 + sl + 1];
                        else
                          {
                            gb[pos[sl]] = b;
                            const double wt = rw[k] * pw[q];
                            if (fp32_weights)
                              gwf[pos[sl]] = static_cast<float>(wt);
                            else
                              gw[pos[sl]] = wt;
                            ++pos[sl];
                          }
                      }
                  }
              }
            for (int s = 0; s < ns; ++s)
              {
                slot_of[c0[s]] = -1;
                grow[b0 + s] = static_cast<int32_t>(I);
              }
          }
      }
      if (outside) return set_error(GLGPU_ERR_ARG, "multigrid: Galerkin product leaves the coarse pattern");
    }
  // blocks on or above the diagonal, and (block, mirror) pairs below it, in block order:
  // counted per coarse row, then written at their offsets on all host threads (a row's
  // columns are sorted, so the mirror is a binary search in row J)
  std::vector<int32_t> &up = T.g_up, &lo = T.g_lo;
  std::vector<int64_t> nup(static_cast<size_t>(ncr) + 1, 0), nlo(static_cast<size_t>(ncr) + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t I = 0; I < ncr; ++I)
    {
      int64_t u = 0;
      for (int32_t b = CP.rowptr[I]; b < CP.rowptr[I + 1]; ++b) u += CP.cols[b] >= I;
      nup[I + 1] = u;
      nlo[I + 1] = (CP.rowptr[I + 1] - CP.rowptr[I]) - u;
    }
  for (int64_t I = 0; I < ncr; ++I)
    {
      nup[I + 1] += nup[I];
      nlo[I + 1] += nlo[I];
    }
  up.assign(static_cast<size_t>(nup[ncr]), 0);
  lo.assign(static_cast<size_t>(2 * nlo[ncr]), 0);
  int asym = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : asym)
  for (int64_t I = 0; I < ncr; ++I)
    {
      int64_t u = nup[I], q = nlo[I];
      for (int32_t b = CP.rowptr[I]; b < CP.rowptr[I + 1]; ++b)
        {
          const int32_t J = CP.cols[b];
          if (J >= I)
            {
              up[u++] = b;
              continue;
            }
          const int32_t *r0 = CP.cols.data() + CP.rowptr[J], *r1 = CP.cols.data() + CP.rowptr[J + 1];
          const int32_t *it = std::lower_bound(r0, r1, static_cast<int32_t>(I));
          if (it == r1 || *it != I) asym = 1;
          lo[2 * q] = b;
          lo[2 * q + 1] = (it != r1 && *it == I) ? static_cast<int32_t>(it - CP.cols.data()) : -1;
          ++q;
        }
    }
  if (asym) return set_error(GLGPU_ERR_ARG, "multigrid: the coarse pattern is not symmetric");
  return GLGPU_OK;
}

} // namespace glgpu

extern "C" glgpu_status glgpu_plan_prolongation(const glgpu_mesh *mesh, int n_inst, int64_t *n_coarse, int64_t *nnz,
                                                int32_t *ptr, int32_t *idx, double *w, double *coarse_xyz)
{
  using namespace glgpu;
  if (!n_coarse || !nnz) return set_error(GLGPU_ERR_ARG, "glgpu_plan_prolongation: n_coarse or nnz is NULL");
  *n_coarse = 0;
  *nnz = 0;
  Plan FP;
  glgpu_status s = build_plan(mesh, n_inst, FP);
  if (s != GLGPU_OK) return s;
  if (FP.dim != 3) return GLGPU_OK;
  std::vector<MgLevel> lv;
  std::string why;
  if (build_hierarchy(mesh, n_inst, 1, lv, why) == 0) return GLGPU_OK;
  std::vector<glgpu_mesh> ms(n_inst);
  for (int k = 0; k < n_inst; ++k)
    {
      const BoxMesh &b = lv[0].meshes[k];
      const bool con = !b.hpar.empty();
      ms[k] = glgpu_mesh{3, b.nn, b.nc, b.xyz.data(), b.cells.data(), b.mask.data(),
                         con ? b.hptr.data() : nullptr, con ? b.hpar.data() : nullptr, con ? b.hw.data() : nullptr};
    }
  Plan CP;
  if ((s = build_plan(ms.data(), n_inst, CP)) != GLGPU_OK) return s;
  TransferTables T;
  if ((s = transfer_tables(mesh, n_inst, lv, 0, FP, CP, T)) != GLGPU_OK) return s;
  *n_coarse = CP.nn;
  *nnz = static_cast<int64_t>(T.pi.size());
  if (ptr) std::copy(T.pp.begin(), T.pp.end(), ptr);
  if (idx) std::copy(T.pi.begin(), T.pi.end(), idx);
  if (w) std::copy(T.pw.begin(), T.pw.end(), w);
  if (coarse_xyz)
    for (int k = 0; k < n_inst; ++k)
      std::copy(lv[0].meshes[k].xyz.begin(), lv[0].meshes[k].xyz.end(), coarse_xyz + 3 * CP.node_off[k]);
  return GLGPU_OK;
}
