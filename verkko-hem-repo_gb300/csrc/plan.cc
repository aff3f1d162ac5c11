// Host-side, once-per-mesh preparation: validation, the condensed block-CSR
// pattern and the per-row assembly plan.  This replaces what the reference does in
// setup_system() with DoFTools::make_sparsity_pattern(dof_handler, sp,
// constraints_newton_update, false) (femgl/src/setup_uniform_B-phase.cc:188-198)
// and what AffineConstraints::distribute_local_to_global decides per cell during
// every assembly (femgl/src/assemble.cc:356-361): here that decision is made once
// and stored as slots, so the device assembly is a gather with no search.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "glgpu_internal.h"

namespace
{
constexpr int kSegLen = 1024; // must not exceed kSegMax of the device kernels
}

namespace glgpu
{
namespace
{
struct Incidence
{
  std::vector<int32_t> ptr;
  bulk_vector<int32_t> cell, loc; // written in full by the fill
};

glgpu_status check_mesh(const glgpu_mesh &m, int k)
{
  const std::string who = "glgpu_create: instance " + std::to_string(k) + ": ";
  if (m.dim != 2 && m.dim != 3) return set_error(GLGPU_ERR_ARG, who + "dim must be 2 or 3");
  if (m.n_nodes <= 0 || m.n_cells <= 0 || !m.xyz || !m.cells) return set_error(GLGPU_ERR_ARG, who + "empty mesh");
  const int nv = 1 << m.dim, B = (m.dim == 3) ? 18 : 2;
  for (int64_t i = 0; i < static_cast<int64_t>(m.n_cells) * nv; ++i)
    if (m.cells[i] < 0 || m.cells[i] >= m.n_nodes) return set_error(GLGPU_ERR_ARG, who + "cell vertex out of range");
  for (int64_t e = 0; e < m.n_cells; ++e)
    {
      const int32_t *c = m.cells + e * nv;
      double h[3] = {1, 1, 1};
      for (int d = 0; d < m.dim; ++d) h[d] = m.xyz[c[nv - 1] * m.dim + d] - m.xyz[c[0] * m.dim + d];
      for (int d = 0; d < m.dim; ++d)
        if (!(h[d] > 0)) return set_error(GLGPU_ERR_ARG, who + "cell is not an axis-aligned box (degenerate edge)");
      for (int v = 0; v < nv; ++v)
        for (int d = 0; d < m.dim; ++d)
          {
            const double expect = m.xyz[c[0] * m.dim + d] + ((v >> d) & 1) * h[d];
            if (std::fabs(m.xyz[c[v] * m.dim + d] - expect) > 1e-9 * (std::fabs(h[d]) + std::fabs(expect)))
              return set_error(GLGPU_ERR_ARG, who + "cell is not an axis-aligned box in deal.II vertex order");
          }
    }
  if (m.dirichlet_mask)
    for (int i = 0; i < m.n_nodes; ++i)
      if (B < 32 && (m.dirichlet_mask[i] >> B) != 0) return set_error(GLGPU_ERR_ARG, who + "mask bit beyond block size");
  if (m.hang_ptr)
    {
      if (m.hang_ptr[0] != 0) return set_error(GLGPU_ERR_ARG, who + "hang_ptr[0] != 0");
      for (int i = 0; i < m.n_nodes; ++i)
        {
          const int np = m.hang_ptr[i + 1] - m.hang_ptr[i];
          if (np < 0 || np > kMaxParents) return set_error(GLGPU_ERR_ARG, who + "bad hanging-constraint row");
          for (int k2 = m.hang_ptr[i]; k2 < m.hang_ptr[i + 1]; ++k2)
            {
              const int p = m.hang_parent[k2];
              if (p < 0 || p >= m.n_nodes || p == i) return set_error(GLGPU_ERR_ARG, who + "bad hanging parent");
              if (m.hang_ptr[p + 1] > m.hang_ptr[p])
                return set_error(GLGPU_ERR_ARG, who + "hanging parent is itself hanging (chains are not supported)");
            }
        }
    }
  return GLGPU_OK;
}
} // namespace

glgpu_status build_plan(const glgpu_mesh *mesh, int n_inst, Plan &P)
{
  if (!mesh || n_inst <= 0) return set_error(GLGPU_ERR_ARG, "glgpu_create: no instances");
  P.dim = mesh[0].dim;
  {
    // instances are validated on all host threads; the first failure is validated again on
    // the calling thread, whose error slot the caller reads
    std::vector<glgpu_status> st(n_inst, GLGPU_OK);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < n_inst; ++k) st[k] = check_mesh(mesh[k], k);
    for (int k = 0; k < n_inst; ++k)
      {
        if (st[k] != GLGPU_OK) return check_mesh(mesh[k], k);
        if (mesh[k].dim != P.dim) return set_error(GLGPU_ERR_ARG, "glgpu_create: all instances must share dim");
      }
  }
  P.B = (P.dim == 3) ? 18 : 2;
  P.nv = 1 << P.dim;
  const int nv = P.nv, B = P.B;
  P.n_inst = n_inst;
  P.node_off.assign(n_inst + 1, 0);
  P.cell_off.assign(n_inst + 1, 0);
  for (int k = 0; k < n_inst; ++k)
    {
      P.node_off[k + 1] = P.node_off[k] + mesh[k].n_nodes;
      P.cell_off[k + 1] = P.cell_off[k] + mesh[k].n_cells;
    }
  P.nn = P.node_off[n_inst];
  P.nc = P.cell_off[n_inst];
  if (P.nn * B >= (int64_t(1) << 31) || P.nc * nv >= (int64_t(1) << 31))
    return set_error(GLGPU_ERR_ARG, "glgpu_create: more than 2^31 dofs in one context; split the batch");
  const int64_t nn = P.nn, nc = P.nc;
  P.cells.resize(nc * nv);
  P.cell_h.resize(nc * 3);
  P.cell_x0.resize(nc * 3);
  P.cell_inst.resize(nc);
  P.node_inst.resize(nn);
  P.mask.assign(nn, 0u);
  P.hptr.assign(nn + 1, 0);
  // instances own disjoint node and cell ranges (their cells reference only their own
  // nodes): the per-instance loops below run on all host threads
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < n_inst; ++k)
    {
      const glgpu_mesh &m = mesh[k];
      const int64_t no = P.node_off[k], co = P.cell_off[k];
      for (int64_t e = 0; e < m.n_cells; ++e)
        {
          const int32_t *c = m.cells + e * nv;
          for (int v = 0; v < nv; ++v) P.cells[(co + e) * nv + v] = static_cast<int32_t>(no + c[v]);
          for (int d = 0; d < 3; ++d)
            {
              P.cell_h[(co + e) * 3 + d] = (d < m.dim) ? m.xyz[c[nv - 1] * m.dim + d] - m.xyz[c[0] * m.dim + d] : 1.0;
              P.cell_x0[(co + e) * 3 + d] = (d < m.dim) ? m.xyz[c[0] * m.dim + d] : 0.0;
            }
          P.cell_inst[co + e] = k;
        }
      for (int64_t i = 0; i < m.n_nodes; ++i)
        {
          P.node_inst[no + i] = k;
          if (m.dirichlet_mask) P.mask[no + i] = m.dirichlet_mask[i];
          P.hptr[no + i + 1] = m.hang_ptr ? (m.hang_ptr[i + 1] - m.hang_ptr[i]) : 0;
        }
    }
  for (int64_t i = 0; i < nn; ++i) P.hptr[i + 1] += P.hptr[i];
  P.hpar.resize(P.hptr[nn]);
  P.hw.resize(P.hptr[nn]);
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < n_inst; ++k)
    {
      const glgpu_mesh &m = mesh[k];
      if (!m.hang_ptr) continue;
      const int64_t no = P.node_off[k];
      for (int64_t i = 0; i < m.n_nodes; ++i)
        for (int j = m.hang_ptr[i]; j < m.hang_ptr[i + 1]; ++j)
          {
            const int64_t dst = P.hptr[no + i] + (j - m.hang_ptr[i]);
            P.hpar[dst] = static_cast<int32_t>(no + m.hang_parent[j]);
            P.hw[dst] = m.hang_weight[j];
          }
    }
  // hanging nodes carry no Dirichlet mask: their constraint takes precedence
  auto hanging = [&](int64_t n) { return P.hptr[n + 1] > P.hptr[n]; };
  for (int64_t i = 0; i < nn; ++i)
    if (hanging(i)) P.mask[i] = 0u;

  // node -> (cell, local vertex) incidence
  // (counting sorts per instance: a node's entries keep ascending cell order)
  Incidence inc;
  inc.ptr.assign(nn + 1, 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < n_inst; ++k)
    for (int64_t e = P.cell_off[k] * nv; e < P.cell_off[k + 1] * nv; ++e) inc.ptr[P.cells[e] + 1]++;
  for (int64_t i = 0; i < nn; ++i) inc.ptr[i + 1] += inc.ptr[i];
  inc.cell.resize(nc * nv);
  inc.loc.resize(nc * nv);
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < n_inst; ++k)
    {
      const int64_t no = P.node_off[k];
      std::vector<int32_t> fill(inc.ptr.begin() + no, inc.ptr.begin() + P.node_off[k + 1]);
      for (int64_t e = P.cell_off[k]; e < P.cell_off[k + 1]; ++e)
        for (int v = 0; v < nv; ++v)
          {
            const int64_t n = P.cells[e * nv + v] - no;
            inc.cell[fill[n]] = static_cast<int32_t>(e);
            inc.loc[fill[n]] = v;
            fill[n]++;
          }
    }
  // parent -> hanging children (parents lie in their child's instance)
  std::vector<int32_t> ch_ptr(nn + 1, 0), ch_node, ch_idx;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < n_inst; ++k)
    for (int64_t i = P.node_off[k]; i < P.node_off[k + 1]; ++i)
      for (int j = P.hptr[i]; j < P.hptr[i + 1]; ++j) ch_ptr[P.hpar[j] + 1]++;
  for (int64_t i = 0; i < nn; ++i) ch_ptr[i + 1] += ch_ptr[i];
  ch_node.resize(ch_ptr[nn]);
  ch_idx.resize(ch_ptr[nn]);
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < n_inst; ++k)
    {
      const int64_t no = P.node_off[k];
      std::vector<int32_t> fill(ch_ptr.begin() + no, ch_ptr.begin() + P.node_off[k + 1]);
      for (int64_t i = no; i < P.node_off[k + 1]; ++i)
        for (int j = P.hptr[i]; j < P.hptr[i + 1]; ++j)
          {
            const int64_t p = P.hpar[j] - no;
            ch_node[fill[p]] = static_cast<int32_t>(i);
            ch_idx[fill[p]] = j;
            fill[p]++;
          }
  }

  // per-row contribution lists and column sets (rows independent)
  struct RowData
  {
    std::vector<int32_t> cols;
    std::vector<int32_t> rc_cell, rc_a;
    std::vector<double> rc_w;
  };
  std::vector<int32_t> row_len(nn, 0), rc_len(nn, 0), ht_len(nn, 0);
  auto gather_row = [&](int64_t n, RowData &R) {
    R.cols.clear();
    R.rc_cell.clear();
    R.rc_a.clear();
    R.rc_w.clear();
    if (hanging(n))
      {
        R.cols.push_back(static_cast<int32_t>(n));
        return;
      }
    auto add_node_contribs = [&](int64_t node, double w) {
      for (int j = inc.ptr[node]; j < inc.ptr[node + 1]; ++j)
        {
          R.rc_cell.push_back(inc.cell[j]);
          R.rc_a.push_back(inc.loc[j]);
          R.rc_w.push_back(w);
        }
    };
    add_node_contribs(n, 1.0);
    for (int j = ch_ptr[n]; j < ch_ptr[n + 1]; ++j) add_node_contribs(ch_node[j], P.hw[ch_idx[j]]);
    for (size_t k = 0; k < R.rc_cell.size(); ++k)
      for (int b = 0; b < nv; ++b)
        {
          const int32_t m = P.cells[static_cast<int64_t>(R.rc_cell[k]) * nv + b];
          if (hanging(m))
            for (int j = P.hptr[m]; j < P.hptr[m + 1]; ++j) R.cols.push_back(P.hpar[j]);
          else
            R.cols.push_back(m);
        }
    if (R.rc_cell.empty()) R.cols.push_back(static_cast<int32_t>(n)); // isolated node: diagonal only
    std::sort(R.cols.begin(), R.cols.end());
    R.cols.erase(std::unique(R.cols.begin(), R.cols.end()), R.cols.end());
  };

#pragma omp parallel
  {
    RowData R;
#pragma omp for schedule(dynamic, 1024)
    for (int64_t n = 0; n < nn; ++n)
      {
        gather_row(n, R);
        row_len[n] = static_cast<int32_t>(R.cols.size());
        rc_len[n] = static_cast<int32_t>(R.rc_cell.size());
        int nh = 0;
        for (size_t k = 0; k < R.rc_cell.size(); ++k)
          for (int b = 0; b < nv; ++b)
            if (hanging(P.cells[static_cast<int64_t>(R.rc_cell[k]) * nv + b])) ++nh;
        ht_len[n] = nh;
      }
  }
  P.rowptr.assign(nn + 1, 0);
  P.rc_ptr.assign(nn + 1, 0);
  std::vector<int64_t> ht_off(nn + 1, 0);
  for (int64_t n = 0; n < nn; ++n)
    {
      P.rowptr[n + 1] = P.rowptr[n] + row_len[n];
      P.rc_ptr[n + 1] = P.rc_ptr[n] + rc_len[n];
      ht_off[n + 1] = ht_off[n] + ht_len[n];
      if (row_len[n] > 32767) return set_error(GLGPU_ERR_ARG, "glgpu_create: row too long");
    }
  P.nnzb = P.rowptr[nn];
  P.max_row_blocks = *std::max_element(row_len.begin(), row_len.end());
  // not zero-filled: the row pass below writes every entry (the lengths come from the pass above)
  P.cols.clear();
  P.cols.resize(P.nnzb);
  P.diag.assign(nn, -1);
  const int64_t nrc = P.rc_ptr[nn];
  P.rc_cell.clear();
  P.rc_a.clear();
  P.rc_w.clear();
  P.rc_slot.clear();
  P.hang_tg.clear();
  P.rc_cell.resize(nrc);
  P.rc_a.resize(nrc);
  P.rc_w.resize(nrc);
  P.rc_slot.resize(nrc * nv);
  P.hang_tg.resize(ht_off[nn]);
  bool bad = false;
#pragma omp parallel
  {
    RowData R;
#pragma omp for schedule(dynamic, 1024)
    for (int64_t n = 0; n < nn; ++n)
      {
        gather_row(n, R);
        std::copy(R.cols.begin(), R.cols.end(), P.cols.begin() + P.rowptr[n]);
        auto slot_of = [&](int32_t col) -> int {
          auto it = std::lower_bound(R.cols.begin(), R.cols.end(), col);
          return (it != R.cols.end() && *it == col) ? static_cast<int>(it - R.cols.begin()) : -1;
        };
        P.diag[n] = P.rowptr[n] + slot_of(static_cast<int32_t>(n));
        int64_t ht = ht_off[n];
        for (size_t k = 0; k < R.rc_cell.size(); ++k)
          {
            const int64_t dst = P.rc_ptr[n] + static_cast<int64_t>(k);
            P.rc_cell[dst] = R.rc_cell[k];
            P.rc_a[dst] = R.rc_a[k];
            P.rc_w[dst] = R.rc_w[k];
            for (int b = 0; b < nv; ++b)
              {
                const int32_t m = P.cells[static_cast<int64_t>(R.rc_cell[k]) * nv + b];
                if (!hanging(m))
                  {
                    const int s = slot_of(m);
                    if (s < 0) bad = true;
                    P.rc_slot[dst * nv + b] = static_cast<int16_t>(s);
                  }
                else
                  {
                    HangTarget &t = P.hang_tg[ht];
                    t.count = P.hptr[m + 1] - P.hptr[m];
                    for (int j = 0; j < kMaxParents; ++j)
                      {
                        t.slot[j] = (j < t.count) ? slot_of(P.hpar[P.hptr[m] + j]) : 0;
                        t.w[j] = (j < t.count) ? P.hw[P.hptr[m] + j] : 0.0;
                        if (j < t.count && t.slot[j] < 0) bad = true;
                      }
                    const int64_t local = ht - ht_off[n];
                    if (local >= 32767) bad = true;
                    P.rc_slot[dst * nv + b] = static_cast<int16_t>(-1 - local);
                    ++ht;
                  }
              }
          }
      }
  }
  if (bad) return set_error(GLGPU_ERR_ARG, "glgpu_create: inconsistent constraint pattern");
  P.ht_off.assign(ht_off.begin(), ht_off.end());
  // regular rows: in the block row of node n, block (a, b) of a cell whose vertex a is n
  // lands in slot 13 + dx + 3 dy + 9 dz, (dx, dy, dz) = bits(b) - bits(a), when the 27
  // columns are the lattice neighbours sorted by node id; verified entry by entry, and
  // the row's eight contributions are then stored in vertex order
  P.reg_rows.clear();
  P.gen_rows.clear();
  P.inst_uniform.assign(n_inst, 1);
  P.inst_h.assign(static_cast<size_t>(n_inst) * 3, 0.0);
  for (int k = 0; k < n_inst; ++k)
    {
      const int64_t c0 = P.cell_off[k], c1 = P.cell_off[k + 1];
      if (c1 <= c0)
        {
          P.inst_uniform[k] = 0;
          continue;
        }
      for (int d = 0; d < 3; ++d) P.inst_h[3 * k + d] = P.cell_h[3 * c0 + d];
      for (int64_t e = c0; e < c1 && P.inst_uniform[k]; ++e)
        for (int d = 0; d < 3; ++d)
          if (P.cell_h[3 * e + d] != P.inst_h[3 * k + d]) P.inst_uniform[k] = 0;
    }
  for (int64_t n = 0; n < nn; ++n)
    {
      bool reg = P.dim == 3 && B == 18 && nv == 8 && row_len[n] == 27 && rc_len[n] == 8 && P.mask[n] == 0 &&
                 P.hptr[n + 1] == P.hptr[n] && P.inst_uniform[P.node_inst[n]];
      unsigned seen = 0;
      for (int k = 0; reg && k < 8; ++k)
        {
          const int64_t r = P.rc_ptr[n] + k;
          const int a = P.rc_a[r];
          if (P.rc_w[r] != 1.0 || (seen >> a) & 1u)
            {
              reg = false;
              break;
            }
          seen |= 1u << a;
          for (int b = 0; b < 8; ++b)
            {
              const int want = 13 + ((b & 1) - (a & 1)) + 3 * (((b >> 1) & 1) - ((a >> 1) & 1)) +
                               9 * (((b >> 2) & 1) - ((a >> 2) & 1));
              if (P.rc_slot[r * nv + b] != want) reg = false;
            }
        }
      if (reg)
        {
          // store the contributions in local-vertex order: contribution a has vertex a
          const int64_t r0 = P.rc_ptr[n];
          int32_t cell[8];
          double w[8];
          int16_t sl[8][8];
          for (int k = 0; k < 8; ++k)
            {
              const int a = P.rc_a[r0 + k];
              cell[a] = P.rc_cell[r0 + k];
              w[a] = P.rc_w[r0 + k];
              for (int b = 0; b < 8; ++b) sl[a][b] = P.rc_slot[(r0 + k) * nv + b];
            }
          for (int a = 0; a < 8; ++a)
            {
              P.rc_cell[r0 + a] = cell[a];
              P.rc_a[r0 + a] = a;
              P.rc_w[r0 + a] = w[a];
              for (int b = 0; b < 8; ++b) P.rc_slot[(r0 + a) * nv + b] = sl[a][b];
            }
        }
      (reg ? P.reg_rows : P.gen_rows).push_back(static_cast<int32_t>(n));
    }
  // reduction segments
  P.seg_len = kSegLen;
  P.seg_begin.clear();
  P.seg_end.clear();
  P.seg_inst.clear();
  P.inst_seg_off.assign(n_inst + 1, 0);
  for (int k = 0; k < n_inst; ++k)
    {
      const int64_t b0 = P.node_off[k] * B, b1 = P.node_off[k + 1] * B;
      for (int64_t s = b0; s < b1; s += P.seg_len)
        {
          P.seg_begin.push_back(s);
          P.seg_end.push_back(std::min<int64_t>(s + P.seg_len, b1));
          P.seg_inst.push_back(k);
        }
      P.inst_seg_off[k + 1] = static_cast<int32_t>(P.seg_begin.size());
    }
  return GLGPU_OK;
}

// A face perpendicular to `axis` is a pair-breaking boundary face when its four vertices lie
// on a boundary plane whose nodes carry the zero-Dirichlet mask of that axis' orbital column
// (setup_uniform_B-phase.cc:134-157 masks exactly the faces with ids 2/3/4).  An unconstrained
// node lies there when its mask holds the column; a hanging node when all its parents do
// (it sits on the edge or face they span).
void robin_faces(const Plan &P, const std::vector<uint8_t> &active, std::vector<uint8_t> &robin)
{
  robin.assign(static_cast<size_t>(P.nc), 0);
  if (P.dim != 3 || P.B != 18) return;
  uint32_t col[3];
  for (int ax = 0; ax < 3; ++ax)
    {
      col[ax] = 0;
      for (int part = 0; part < 2; ++part)
        for (int mu = 0; mu < 3; ++mu) col[ax] |= 1u << (9 * part + 3 * mu + ax);
    }
  auto on_plane = [&](int32_t n, int ax) {
    const int32_t h0 = P.hptr[n], h1 = P.hptr[n + 1];
    if (h1 == h0) return (P.mask[n] & col[ax]) == col[ax];
    for (int32_t k = h0; k < h1; ++k)
      if ((P.mask[P.hpar[k]] & col[ax]) != col[ax]) return false;
    return true;
  };
  for (int64_t e = 0; e < P.nc; ++e)
    {
      if (!active[P.cell_inst[e]]) continue;
      const int32_t *cv = &P.cells[8 * e];
      uint8_t bits = 0;
      for (int f = 0; f < 6; ++f)
        {
          const int ax = f / 2, side = f % 2;
          bool ok = true;
          for (int v = 0; v < 8 && ok; ++v)
            if (((v >> ax) & 1) == side && !on_plane(cv[v], ax)) ok = false;
          if (ok) bits |= static_cast<uint8_t>(1u << f);
        }
      robin[e] = bits;
    }
}

} // namespace glgpu

using namespace glgpu;

extern "C" glgpu_status glgpu_plan_info(const glgpu_mesh *mesh, int n_inst, int64_t *info)
{
  if (!info) return set_error(GLGPU_ERR_ARG, "glgpu_plan_info: info is NULL");
  Plan P;
  glgpu_status s = build_plan(mesh, n_inst, P);
  if (s != GLGPU_OK) return s;
  info[0] = P.nn;
  info[1] = P.nnzb;
  info[2] = P.max_row_blocks;
  info[3] = static_cast<int64_t>(P.rc_cell.size());
  info[4] = static_cast<int64_t>(P.hang_tg.size());
  info[5] = static_cast<int64_t>(P.seg_begin.size());
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_plan_robin(const glgpu_mesh *mesh, int n_inst, uint8_t *faces)
{
  if (!faces) return set_error(GLGPU_ERR_ARG, "glgpu_plan_robin: faces is NULL");
  Plan P;
  glgpu_status s = build_plan(mesh, n_inst, P);
  if (s != GLGPU_OK) return s;
  std::vector<uint8_t> robin;
  robin_faces(P, std::vector<uint8_t>(static_cast<size_t>(n_inst), 1), robin);
  std::memcpy(faces, robin.data(), robin.size());
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_plan_pattern(const glgpu_mesh *mesh, int n_inst, int32_t *rowptr, int32_t *cols)
{
  Plan P;
  glgpu_status s = build_plan(mesh, n_inst, P);
  if (s != GLGPU_OK) return s;
  if (rowptr) std::memcpy(rowptr, P.rowptr.data(), sizeof(int32_t) * P.rowptr.size());
  if (cols) std::memcpy(cols, P.cols.data(), sizeof(int32_t) * P.cols.size());
  return GLGPU_OK;
}
