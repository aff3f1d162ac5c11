// Host side of the GPU Kelly error estimator: the interior face pairs of a mesh of
// axis-aligned hexahedra with at most one level of refinement difference across a face
// (the reference estimates with deal.II's KellyErrorEstimator, femgl/src/refine.cc:147-157).
//
// A face is keyed by its four vertices after periodic identification (a node constrained to a
// single parent with weight 1 stands for that parent; constrained nodes with the same
// constraint row, a hanging node and its periodic image, stand for one node).  Two faces with the same key are a
// conforming pair.  A face that contains a hanging node with four parents is a quarter of
// the coarse face spanned by those parents and pairs with the cell owning that coarse face.
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <vector>

#include "glgpu_internal.h"

namespace glgpu
{
glgpu_status kelly_faces(const Plan &P, KellyFaces &out)
{
  out = KellyFaces{};
  if (P.dim != 3 || P.nv != 8) return set_error(GLGPU_ERR_ARG, "error estimator: 3D hexahedral meshes only");
  // node identity modulo periodicity: a node constrained to one parent with weight 1 is that
  // parent; other constrained nodes with identical constraint rows (a hanging node and its
  // periodic image) share the smallest such node id
  std::map<std::vector<std::pair<int32_t, double>>, int32_t> row_id;
  std::vector<int32_t> canon(P.nn);
  for (int64_t n = 0; n < P.nn; ++n)
    {
      const int32_t h0 = P.hptr[n], h1 = P.hptr[n + 1];
      if (h1 == h0)
        canon[n] = static_cast<int32_t>(n);
      else if (h1 - h0 == 1 && P.hw[h0] == 1.0)
        canon[n] = P.hpar[h0];
      else
        {
          std::vector<std::pair<int32_t, double>> row;
          for (int32_t k = h0; k < h1; ++k) row.push_back({P.hpar[k], P.hw[k]});
          auto it = row_id.emplace(row, static_cast<int32_t>(n)).first;
          canon[n] = it->second;
        }
    }
  auto resolve = [&](int32_t n) { return canon[n]; };
  using Key = std::array<int32_t, 4>;
  std::map<Key, std::vector<std::pair<int32_t, int>>> whole;  // key -> (cell, face)
  std::vector<std::pair<Key, std::pair<int32_t, int>>> quarter; // coarse key -> fine (cell, face)
  for (int64_t e = 0; e < P.nc; ++e)
    for (int f = 0; f < 6; ++f)
      {
        const int ax = f / 2, side = f % 2;
        Key k;
        int nk = 0;
        int32_t center = -1;
        for (int v = 0; v < 8; ++v)
          if (((v >> ax) & 1) == side)
            {
              const int32_t n = P.cells[8 * e + v];
              k[nk++] = resolve(n);
              if (P.hptr[n + 1] - P.hptr[n] == 4) center = n;
            }
        std::sort(k.begin(), k.end());
        whole[k].push_back({static_cast<int32_t>(e), f});
        if (center >= 0)
          {
            Key c;
            for (int j = 0; j < 4; ++j) c[j] = P.hpar[P.hptr[center] + j];
            std::sort(c.begin(), c.end());
            quarter.push_back({c, {static_cast<int32_t>(e), f}});
          }
      }
  auto tangential = [](int ax, int &t1, int &t2) {
    t1 = (ax == 0) ? 1 : 0;
    t2 = (ax == 2) ? 1 : 2;
  };
  auto add = [&](int32_t a, int fa, int32_t b, int fb, int sub) {
    int ob = 0;
    if (sub)
      {
        int t1, t2;
        tangential(fa / 2, t1, t2);
        const int ts[2] = {t1, t2};
        for (int j = 0; j < 2; ++j)
          {
            const double off = (P.cell_x0[3 * a + ts[j]] - P.cell_x0[3 * b + ts[j]]) / P.cell_h[3 * a + ts[j]];
            const long o = std::lround(off);
            if ((o != 0 && o != 1) || std::fabs(off - o) > 1e-6) return false;
            ob |= static_cast<int>(o) << j;
          }
      }
    out.a.push_back(a);
    out.b.push_back(b);
    out.fa.push_back(static_cast<int8_t>(fa));
    out.fb.push_back(static_cast<int8_t>(fb));
    out.ob.push_back(static_cast<int8_t>(ob));
    out.sub.push_back(static_cast<int8_t>(sub));
    return true;
  };
  for (const auto &kv : whole)
    {
      const auto &v = kv.second;
      if (v.size() == 2)
        {
          if (v[0].second / 2 != v[1].second / 2 || v[0].second == v[1].second)
            return set_error(GLGPU_ERR_ARG, "error estimator: faces with one key do not face each other");
          add(v[0].first, v[0].second, v[1].first, v[1].second, 0);
        }
      else if (v.size() > 2)
        return set_error(GLGPU_ERR_ARG, "error estimator: a face shared by more than two cells");
    }
  for (const auto &q : quarter)
    {
      auto it = whole.find(q.first);
      if (it == whole.end()) continue; // the parents span no cell face: not a coarse-fine face
      const int32_t b = it->second[0].first;
      const int fb = it->second[0].second;
      // a fine face perpendicular to the coarse face also touches its centre node; it is an
      // interior fine-fine face, paired above
      if (fb / 2 != q.second.second / 2) continue;
      if (it->second.size() != 1)
        return set_error(GLGPU_ERR_ARG, "error estimator: a refined face has more than one coarse neighbour");
      if (!add(q.second.first, q.second.second, b, fb, 1))
        return set_error(GLGPU_ERR_ARG, "error estimator: only one level of refinement across a face is supported");
    }
  // per cell: the pairs it takes part in, in pair order
  const int64_t np = static_cast<int64_t>(out.a.size());
  out.cell_ptr.assign(P.nc + 1, 0);
  for (int64_t k = 0; k < np; ++k)
    {
      out.cell_ptr[out.a[k] + 1]++;
      out.cell_ptr[out.b[k] + 1]++;
    }
  for (int64_t e = 0; e < P.nc; ++e) out.cell_ptr[e + 1] += out.cell_ptr[e];
  out.cell_pair.resize(out.cell_ptr[P.nc]);
  std::vector<int32_t> fill(out.cell_ptr.begin(), out.cell_ptr.end() - 1);
  for (int64_t k = 0; k < np; ++k)
    {
      out.cell_pair[fill[out.a[k]]++] = static_cast<int32_t>(k);
      out.cell_pair[fill[out.b[k]]++] = static_cast<int32_t>(k);
    }
  return GLGPU_OK;
}

} // namespace glgpu

using namespace glgpu;

extern "C" glgpu_status glgpu_plan_kelly(const glgpu_mesh *mesh, int n_inst, int64_t *n_pairs, int32_t *a, int8_t *fa,
                                         int32_t *b, int8_t *fb, int8_t *sub)
{
  if (!n_pairs) return set_error(GLGPU_ERR_ARG, "glgpu_plan_kelly: n_pairs is NULL");
  Plan P;
  glgpu_status s = build_plan(mesh, n_inst, P);
  if (s != GLGPU_OK) return s;
  KellyFaces F;
  if ((s = kelly_faces(P, F)) != GLGPU_OK) return s;
  const size_t np = F.a.size();
  *n_pairs = static_cast<int64_t>(np);
  for (size_t k = 0; k < np; ++k)
    {
      if (a) a[k] = F.a[k];
      if (fa) fa[k] = F.fa[k];
      if (b) b[k] = F.b[k];
      if (fb) fb[k] = F.fb[k];
      if (sub) sub[k] = F.sub[k];
    }
  return GLGPU_OK;
}
