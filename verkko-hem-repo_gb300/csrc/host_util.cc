// Host-side helpers of the C ABI: material parameters, structured box meshes with
// one level of refinement, and the B-phase initial guess.  No device work here.
#include <algorithm>
#include <functional>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "glgpu.h"
#include "glgpu_internal.h"

namespace glgpu
{
// ---------------------------------------------------------------------------------
// Matep: strong-coupling Ginzburg-Landau coefficients, restated from the reference
// matep/src/matep.cc:46-206 and :213-333.  The tables are the reference's data
// (Wiman-Sauls strong-coupling coefficients and Tc(p) on a 2-bar grid, matep.cc:59-65);
// the arithmetic reproduces the reference's mix of float constants, float
// interpolation results and double arithmetic, so results are bit-identical.
// ---------------------------------------------------------------------------------
namespace
{
const double kC1[18] = {-0.0098, -0.0127, -0.0155, -0.0181, -0.0207, -0.0231, -0.0254, -0.0275, -0.0295,
                        -0.0314, -0.0330, -0.0345, -0.0358, -0.0370, -0.0381, -0.0391, -0.0402, -0.0413};
const double kC2[18] = {-0.0419, -0.0490, -0.0562, -0.0636, -0.0711, -0.0786, -0.0861, -0.0936, -0.1011,
                        -0.1086, -0.1160, -0.1233, -0.1306, -0.1378, -0.1448, -0.1517, -0.1583, -0.1645};
const double kC3[18] = {-0.0132, -0.0161, -0.0184, -0.0202, -0.0216, -0.0226, -0.0233, -0.0239, -0.0243,
                        -0.0247, -0.0249, -0.0252, -0.0255, -0.0258, -0.0262, -0.0265, -0.0267, -0.0268};
const double kC4[18] = {-0.0047, -0.0276, -0.0514, -0.0760, -0.1010, -0.1260, -0.1508, -0.1751, -0.1985,
                        -0.2208, -0.2419, -0.2614, -0.2795, -0.2961, -0.3114, -0.3255, -0.3388, -0.3518};
const double kC5[18] = {-0.0899, -0.1277, -0.1602, -0.1880, -0.2119, -0.2324, -0.2503, -0.2660, -0.2801,
                        -0.2930, -0.3051, -0.3167, -0.3280, -0.3392, -0.3502, -0.3611, -0.3717, -0.3815};
const double kTc[18] = {0.929, 1.181, 1.388, 1.560, 1.705, 1.828, 1.934, 2.026, 2.106,
                        2.177, 2.239, 2.293, 2.339, 2.378, 2.411, 2.438, 2.463, 2.486};

// pi and zeta(3) are single-precision literals widened to double in the reference.
const double kPi = static_cast<double>(3.14159265358979323846264338328f);
const double kZeta3 = static_cast<double>(1.2020569031595942f);

double c_beta() { return (7.0 * kZeta3) / (80.0 * kPi * kPi); }

// Piecewise-linear interpolation on the 2-bar grid; the value is rounded to float.
double interp(const double *tab, double p)
{
  const int k = static_cast<int>(std::floor(p / 2.0));
  const float pk = static_cast<float>(2 * k);
  const float v = static_cast<float>(((tab[k + 1] - tab[k]) / 2.0) * (p - pk) + tab[k]);
  return static_cast<double>(v);
}
} // namespace

int matep_eval(double p, double t, bool scc, double *out)
{
  if (!(p >= 0.0 && p < 34.0) || !std::isfinite(t)) return -1;
  const double cb = c_beta();
  const double alpha = 1.0 * (t - 1.0);
  double b[5];
  const double base[5] = {-1.0, 2.0, 2.0, 2.0, -2.0};
  const double *tabs[5] = {kC1, kC2, kC3, kC4, kC5};
  for (int i = 0; i < 5; ++i) b[i] = scc ? cb * (base[i] + t * interp(tabs[i], p)) : cb * base[i];
  const double bA = b[1] + b[3] + b[4];
  const double bB = b[0] + b[1] + static_cast<double>(1.f / 3.f) * (b[2] + b[3] + b[4]);
  out[0] = alpha;
  for (int i = 0; i < 5; ++i) out[1 + i] = b[i];
  out[6] = (t <= 1.0) ? std::sqrt(-alpha / (2.0 * bA)) : 0.0;
  out[7] = (t <= 1.0) ? std::sqrt(-alpha / (2.0 * bB)) : 0.0;
  out[8] = interp(kTc, p);
  out[9] = (t <= 1.0) ? static_cast<double>(-1.f / 4.f) * std::pow(alpha, 2.0) / bA : 0.0;
  out[10] = (t <= 1.0) ? static_cast<double>(-1.f / 4.f) * std::pow(alpha, 2.0) / bB : 0.0;
  out[11] = bA;
  out[12] = bB;
  return 0;
}

// ---------------------------------------------------------------------------------
// Box mesh.  Lattice coordinates are in units of half a coarse cell; nodes are
// numbered by lattice (z, y, x), cells by the lattice of their first vertex.
// ---------------------------------------------------------------------------------
int mesh_box(const double *lo, const double *hi, const int *n, double band, const int *dir3, BoxMesh &m,
             const int8_t *refine)
{
  const int nx = n[0], ny = n[1], nz = n[2];
  if (nx < 1 || ny < 1 || nz < 1) return -1;
  if (dir3)
    for (int d = 0; d < 2; ++d)
      if (dir3[d] < 0 || dir3[d] > 2) return -1;
  double h[3];
  for (int d = 0; d < 3; ++d)
    {
      h[d] = (hi[d] - lo[d]) / n[d];
      if (!(h[d] > 0)) return -1;
    }
  const int64_t Lx = 2 * nx + 1, Ly = 2 * ny + 1, Lz = 2 * nz + 1;
  std::vector<char> fine_layer(nz, 0);
  for (int k = 0; k < nz; ++k)
    {
      const double zc = lo[2] + (k + 0.5) * h[2];
      fine_layer[k] = (std::fabs(zc - lo[2]) < band) || (std::fabs(hi[2] - zc) < band);
    }
  struct C
  {
    int64_t key;
    int32_t b[3];
    int32_t s;
  };
  std::vector<C> cl;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        {
          if (refine ? refine[(static_cast<int64_t>(k) * ny + j) * nx + i] > 0 : fine_layer[k] != 0)
            for (int dk = 0; dk < 2; ++dk)
              for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di)
                  {
                    C c{0, {2 * i + di, 2 * j + dj, 2 * k + dk}, 1};
                    c.key = (c.b[2] * Ly + c.b[1]) * Lx + c.b[0];
                    cl.push_back(c);
                  }
          else
            {
              C c{0, {2 * i, 2 * j, 2 * k}, 2};
              c.key = (c.b[2] * Ly + c.b[1]) * Lx + c.b[0];
              cl.push_back(c);
            }
        }
  std::sort(cl.begin(), cl.end(), [](const C &a, const C &b) { return a.key < b.key; });
  const int64_t ncell = static_cast<int64_t>(cl.size());
  std::vector<int64_t> vkey(ncell * 8);
  for (int64_t e = 0; e < ncell; ++e)
    for (int v = 0; v < 8; ++v)
      {
        const int64_t x = cl[e].b[0] + ((v >> 0) & 1) * cl[e].s, y = cl[e].b[1] + ((v >> 1) & 1) * cl[e].s,
                      z = cl[e].b[2] + ((v >> 2) & 1) * cl[e].s;
        vkey[e * 8 + v] = (z * Ly + y) * Lx + x;
      }
  std::vector<int64_t> ukey(vkey);
  std::sort(ukey.begin(), ukey.end());
  ukey.erase(std::unique(ukey.begin(), ukey.end()), ukey.end());
  const int64_t nn = static_cast<int64_t>(ukey.size());
  if (nn > INT32_MAX / 32 || ncell > INT32_MAX / 8) return -1;
  auto nid = [&](int64_t x, int64_t y, int64_t z) -> int64_t {
    if (x < 0 || y < 0 || z < 0 || x >= Lx || y >= Ly || z >= Lz) return -1;
    const int64_t key = (z * Ly + y) * Lx + x;
    auto it = std::lower_bound(ukey.begin(), ukey.end(), key);
    return (it != ukey.end() && *it == key) ? (it - ukey.begin()) : -1;
  };
  m.nn = static_cast<int>(nn);
  m.nc = static_cast<int>(ncell);
  m.xyz.resize(nn * 3);
  for (int64_t i = 0; i < nn; ++i)
    {
      const int64_t key = ukey[i];
      const int64_t x = key % Lx, y = (key / Lx) % Ly, z = key / (Lx * Ly);
      m.xyz[3 * i + 0] = lo[0] + x * (h[0] * 0.5);
      m.xyz[3 * i + 1] = lo[1] + y * (h[1] * 0.5);
      m.xyz[3 * i + 2] = lo[2] + z * (h[2] * 0.5);
    }
  m.cells.resize(ncell * 8);
  for (int64_t e = 0; e < ncell * 8; ++e)
    m.cells[e] = static_cast<int32_t>(std::lower_bound(ukey.begin(), ukey.end(), vkey[e]) - ukey.begin());

  // hanging nodes on faces of coarse cells (none unless some cell was refined)
  std::vector<int32_t> npar(nn, 0);
  std::vector<int32_t> par(nn * 4, -1);
  std::vector<double> wt(nn * 4, 0.0);
  bool any_refined = false;
  for (int64_t e = 0; e < ncell && !any_refined; ++e) any_refined = cl[e].s == 1;
  for (int64_t e = 0; e < ncell && any_refined; ++e)
    {
      if (cl[e].s != 2) continue;
      const int32_t *b = cl[e].b;
      for (int axis = 0; axis < 3; ++axis)
        for (int side = 0; side < 2; ++side)
          {
            int ta = (axis == 0) ? 1 : 0, tb = (axis == 2) ? 1 : 2;
            for (int u = 0; u < 3; ++u)
              for (int v = 0; v < 3; ++v)
                {
                  if (u != 1 && v != 1) continue;
                  int64_t p[3] = {b[0], b[1], b[2]};
                  p[axis] += 2 * side;
                  p[ta] += u;
                  p[tb] += v;
                  const int64_t id = nid(p[0], p[1], p[2]);
                  if (id < 0 || npar[id] > 0) continue;
                  std::vector<int64_t> ps;
                  if (u == 1 && v == 1)
                    {
                      for (int uu = 0; uu <= 2; uu += 2)
                        for (int vv = 0; vv <= 2; vv += 2)
                          {
                            int64_t q[3] = {b[0], b[1], b[2]};
                            q[axis] += 2 * side;
                            q[ta] += uu;
                            q[tb] += vv;
                            ps.push_back(nid(q[0], q[1], q[2]));
                          }
                    }
                  else
                    {
                      int64_t q1[3] = {p[0], p[1], p[2]}, q2[3] = {p[0], p[1], p[2]};
                      const int t = (u == 1) ? ta : tb;
                      q1[t] -= 1;
                      q2[t] += 1;
                      ps.push_back(nid(q1[0], q1[1], q1[2]));
                      ps.push_back(nid(q2[0], q2[1], q2[2]));
                    }
                  std::sort(ps.begin(), ps.end());
                  const double w = 1.0 / static_cast<double>(ps.size());
                  for (size_t k = 0; k < ps.size(); ++k)
                    {
                      if (ps[k] < 0) return -2;
                      par[id * 4 + k] = static_cast<int32_t>(ps[k]);
                      wt[id * 4 + k] = w;
                    }
                  npar[id] = static_cast<int32_t>(ps.size());
                }
          }
    }
  // periodic axes: the upper face's nodes are constrained to their images on the lower face;
  // then every constraint is resolved to unconstrained parents (weights multiply, repeated
  // parents add, parents sorted)
  const bool per[2] = {dir3 && dir3[0] == 2, dir3 && dir3[1] == 2};
  if (per[0] || per[1])
    {
      const int64_t Lp[2] = {Lx, Ly};
      std::vector<std::vector<std::pair<int32_t, double>>> raw(nn);
      for (int64_t i = 0; i < nn; ++i)
        for (int k = 0; k < npar[i]; ++k) raw[i].push_back({par[i * 4 + k], wt[i * 4 + k]});
      for (int axis = 0; axis < 2; ++axis)
        if (per[axis])
          for (int64_t i = 0; i < nn; ++i)
            {
              const int64_t key = ukey[i];
              int64_t c3[3] = {key % Lx, (key / Lx) % Ly, key / (Lx * Ly)};
              if (c3[axis] == 0)
                {
                  // the two faces must carry the same nodes
                  c3[axis] = Lp[axis] - 1;
                  if (nid(c3[0], c3[1], c3[2]) < 0) return -2;
                  continue;
                }
              if (c3[axis] != Lp[axis] - 1) continue;
              c3[axis] = 0;
              const int64_t img = nid(c3[0], c3[1], c3[2]);
              if (img < 0) return -2;
              raw[i].assign(1, {static_cast<int32_t>(img), 1.0});
            }
      std::vector<std::vector<std::pair<int32_t, double>>> res(nn);
      std::vector<char> done(nn, 0);
      // images lie on lower faces and hanging parents on coarse vertices, so the
      // substitution terminates; depth is bounded by two periodic steps and one hanging step
      std::function<const std::vector<std::pair<int32_t, double>> &(int64_t, int)> resolve =
        [&](int64_t i, int depth) -> const std::vector<std::pair<int32_t, double>> & {
        if (!done[i])
          {
            std::vector<std::pair<int32_t, double>> out;
            if (raw[i].empty())
              out.push_back({static_cast<int32_t>(i), 1.0});
            else if (depth < 8)
              for (const auto &pw : raw[i])
                for (const auto &qw : resolve(pw.first, depth + 1)) out.push_back({qw.first, pw.second * qw.second});
            std::sort(out.begin(), out.end());
            std::vector<std::pair<int32_t, double>> merged;
            for (const auto &t : out)
              if (!merged.empty() && merged.back().first == t.first)
                merged.back().second += t.second;
              else
                merged.push_back(t);
            res[i] = std::move(merged);
            done[i] = 1;
          }
        return res[i];
      };
      for (int64_t i = 0; i < nn; ++i)
        {
          npar[i] = 0;
          if (raw[i].empty()) continue;
          const auto &r = resolve(i, 0);
          if (r.empty() || r.size() > 4) return -2;
          for (size_t k = 0; k < r.size(); ++k)
            {
              if (!raw[r[k].first].empty()) return -2;
              par[i * 4 + k] = r[k].first;
              wt[i * 4 + k] = r[k].second;
            }
          npar[i] = static_cast<int32_t>(r.size());
        }
    }
  m.hptr.assign(nn + 1, 0);
  for (int64_t i = 0; i < nn; ++i) m.hptr[i + 1] = m.hptr[i] + npar[i];
  m.hpar.resize(m.hptr[nn]);
  m.hw.resize(m.hptr[nn]);
  for (int64_t i = 0; i < nn; ++i)
    for (int k = 0; k < npar[i]; ++k)
      {
        m.hpar[m.hptr[i] + k] = par[i * 4 + k];
        m.hw[m.hptr[i] + k] = wt[i * 4 + k];
      }
  // zero-Dirichlet masks: orbital column `axis` of u and v on that axis' faces
  m.mask.assign(nn, 0u);
  const bool on[3] = {dir3 && dir3[0] == 1, dir3 && dir3[1] == 1, !dir3 || dir3[2] != 0};
  const int64_t Ls[3] = {Lx, Ly, Lz};
  for (int64_t i = 0; i < nn; ++i)
    {
      if (npar[i] > 0) continue;
      const int64_t key = ukey[i];
      const int64_t c3[3] = {key % Lx, (key / Lx) % Ly, key / (Lx * Ly)};
      for (int axis = 0; axis < 3; ++axis)
        if (on[axis] && (c3[axis] == 0 || c3[axis] == Ls[axis] - 1)) m.mask[i] |= column_mask(axis);
    }
  return 0;
}

// splitmix64: counter-based, so every dof's draw depends only on (seed, index).
static inline uint64_t mix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double gaussian(uint64_t seed, uint64_t index)
{
  const uint64_t a = mix64(seed * 0x632BE59BD9B4E019ull + 2 * index);
  const uint64_t b = mix64(seed * 0x632BE59BD9B4E019ull + 2 * index + 1);
  const double u1 = (static_cast<double>(a >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double u2 = static_cast<double>(b >> 11) * (1.0 / 9007199254740992.0);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

// Weak-coupling pair-density-wave initial state (femgl/inc/pdw_config.h:111-298, set up by
// setup_weak-coupling-PDW-configuration.cc:286-320): the B phase gap/sqrt(3) on the diagonal
// of u plus a modulation of amplitude gap * u built from four fitted profiles across the
// slab (argument s = (z + half_D) / D in [0, 1]) and the hexagonal harmonics of wave number
// q = pi / (sqrt(3) D) in the plane.  The profile coefficients are the reference's fits.
namespace
{
double horner(const double *c, int n, double s)
{
  double v = 0.0;
  for (int k = n - 1; k >= 0; --k) v = v * s + c[k];
  return v;
}
const double kPdwF1[7] = {-0.010674533968153196, -0.04928146307995591, 0.4123298769345518, -5.957210687551436,
                          15.697110273856326,    -14.963347649994844,  4.860888318571941};
const double kPdwF2[10] = {0.005381764646081998, -0.09659207269737603, 3.059717163195402, -35.01132629189211,
                           193.9107091164305,    -594.3817533999686,   1058.3851407510472, -1088.4440880311813,
                           599.3158862587954,    -136.74038236803835};
const double kPdwF3[8] = {-0.008476309862633497, -0.15843411116780842, 1.1880072170146772, -8.79341508668322,
                          32.93035389045762,     -56.473628486426286,  44.90526146438388,  -13.60443812339298};
const double kPdwF4[4] = {0.703221673991666, 0.07213025175696147, -4.458423083418102, 2.9780246543754445};
} // namespace

void pdw_state(double gap, double u, double half_D, double x, double y, double z, double *a)
{
  const double D = 2.0 * half_D, q = 3.141592653589793 / (1.7320508075688772 * D);
  const double s = (z + half_D) / D;
  const double f1 = horner(kPdwF1, 7, s), f2 = horner(kPdwF2, 10, s), f3 = horner(kPdwF3, 8, s),
               f4 = horner(kPdwF4, 4, s);
  const double r2 = std::sqrt(2.0), r3 = std::sqrt(3.0), r6 = std::sqrt(6.0);
  const double cx = std::cos(q * x), hx_c = std::cos(0.5 * q * x), hx_s = std::sin(0.5 * q * x);
  const double hy_c = std::cos(0.5 * r3 * q * y), hy_s = std::sin(0.5 * r3 * q * y);
  const double c1 = cx - hx_c * hy_c;             // cos qx - cos(qx/2) cos(sqrt3 qy/2)
  const double c2 = cx + 2.0 * hx_c * hy_c;       // cos qx + 2 cos(qx/2) cos(sqrt3 qy/2)
  const double s1 = hx_s * hy_s;                  // sin(qx/2) sin(sqrt3 qy/2)
  const double s2 = hy_c * hx_s + std::sin(q * x); // cos(sqrt3 qy/2) sin(qx/2) + sin qx
  const double s3 = hx_c * hy_s;                  // cos(qx/2) sin(sqrt3 qy/2)
  const double b = gap / r3, g = gap * u;
  for (int c = 0; c < 18; ++c) a[c] = 0.0;
  a[0] = b + g * (2.0 * f1 + 2.0 * f2 * c1);
  a[1] = g * (2.0 * f1 - 2.0 * r3 * f2 * s1);
  a[2] = g * (2.0 * f1 + 2.0 * r2 * f3 * s2);
  a[3] = g * (2.0 * r3 * f1 * c2 - 2.0 * r3 * f2 * s1);
  a[4] = b + g * (-2.0 * f2 * c1 + 2.0 * r3 * f1 * c2);
  a[5] = g * (2.0 * r3 * f1 * c2 + 2.0 * r6 * f3 * s3);
  a[6] = g * (2.0 * r2 * f4 * s2);
  a[7] = g * (2.0 * r6 * f4 * s3);
  a[8] = b;
}

} // namespace glgpu

using namespace glgpu;

extern "C" glgpu_status glgpu_matep(double p, double t, int scc, double *out)
{
  if (!out) return set_error(GLGPU_ERR_ARG, "glgpu_matep: out is NULL");
  if (matep_eval(p, t, scc != 0, out) != 0)
    return set_error(GLGPU_ERR_ARG, "glgpu_matep: pressure outside [0, 34) bar or non-finite t");
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_mesh_box(const double *lo, const double *hi, const int *n, double refine_band,
                                       const int *dirichlet_xy, int *n_nodes, int *n_cells, int *n_hang_entries,
                                       double *xyz, int32_t *cells, uint32_t *mask, int32_t *hang_ptr,
                                       int32_t *hang_parent, double *hang_weight)
{
  if (!lo || !hi || !n) return set_error(GLGPU_ERR_ARG, "glgpu_mesh_box: NULL argument");
  BoxMesh m;
  const int dir3[3] = {dirichlet_xy ? dirichlet_xy[0] : 0, dirichlet_xy ? dirichlet_xy[1] : 0, 1};
  const int rc = mesh_box(lo, hi, n, refine_band, dir3, m);
  if (rc != 0) return set_error(GLGPU_ERR_ARG, "glgpu_mesh_box: invalid box or mesh too large");
  if (n_nodes) *n_nodes = m.nn;
  if (n_cells) *n_cells = m.nc;
  if (n_hang_entries) *n_hang_entries = static_cast<int>(m.hpar.size());
  if (xyz) std::memcpy(xyz, m.xyz.data(), sizeof(double) * m.xyz.size());
  if (cells) std::memcpy(cells, m.cells.data(), sizeof(int32_t) * m.cells.size());
  if (mask) std::memcpy(mask, m.mask.data(), sizeof(uint32_t) * m.mask.size());
  if (hang_ptr) std::memcpy(hang_ptr, m.hptr.data(), sizeof(int32_t) * m.hptr.size());
  if (hang_parent && !m.hpar.empty()) std::memcpy(hang_parent, m.hpar.data(), sizeof(int32_t) * m.hpar.size());
  if (hang_weight && !m.hw.empty()) std::memcpy(hang_weight, m.hw.data(), sizeof(double) * m.hw.size());
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_pdw_guess(double p, double t, int scc, double u, double half_D, int n_nodes,
                                        const double *xyz, double *x)
{
  if (!x || !xyz || n_nodes < 0 || !(half_D > 0.0)) return set_error(GLGPU_ERR_ARG, "glgpu_pdw_guess: bad argument");
  double mp[13];
  if (matep_eval(p, t, scc != 0, mp) != 0) return set_error(GLGPU_ERR_ARG, "glgpu_pdw_guess: bad (p, t)");
  for (int64_t i = 0; i < static_cast<int64_t>(n_nodes); ++i)
    pdw_state(mp[7], u, half_D, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], x + 18 * i);
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_mesh_box_refine(const double *lo, const double *hi, const int *n, const int8_t *flags,
                                              const int *dirichlet_xy, int *n_nodes, int *n_cells,
                                              int *n_hang_entries, double *xyz, int32_t *cells, uint32_t *mask,
                                              int32_t *hang_ptr, int32_t *hang_parent, double *hang_weight)
{
  if (!lo || !hi || !n || !flags) return set_error(GLGPU_ERR_ARG, "glgpu_mesh_box_refine: NULL argument");
  BoxMesh m;
  const int dir3[3] = {dirichlet_xy ? dirichlet_xy[0] : 0, dirichlet_xy ? dirichlet_xy[1] : 0, 1};
  const int rc = mesh_box(lo, hi, n, 0.0, dir3, m, flags);
  if (rc == -2)
    return set_error(GLGPU_ERR_ARG, "glgpu_mesh_box_refine: refinement differs across a periodic face pair");
  if (rc != 0) return set_error(GLGPU_ERR_ARG, "glgpu_mesh_box_refine: invalid box or mesh too large");
  if (n_nodes) *n_nodes = m.nn;
  if (n_cells) *n_cells = m.nc;
  if (n_hang_entries) *n_hang_entries = static_cast<int>(m.hpar.size());
  if (xyz) std::memcpy(xyz, m.xyz.data(), sizeof(double) * m.xyz.size());
  if (cells) std::memcpy(cells, m.cells.data(), sizeof(int32_t) * m.cells.size());
  if (mask) std::memcpy(mask, m.mask.data(), sizeof(uint32_t) * m.mask.size());
  if (hang_ptr) std::memcpy(hang_ptr, m.hptr.data(), sizeof(int32_t) * m.hptr.size());
  if (hang_parent && !m.hpar.empty()) std::memcpy(hang_parent, m.hpar.data(), sizeof(int32_t) * m.hpar.size());
  if (hang_weight && !m.hw.empty()) std::memcpy(hang_weight, m.hw.data(), sizeof(double) * m.hw.size());
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_box_interpolate(const double *lo, const double *hi, const int *n, const double *x_box,
                                              int n_points, const double *xyz, double *x)
{
  if (!lo || !hi || !n || !x_box || !xyz || !x || n_points < 0)
    return set_error(GLGPU_ERR_ARG, "glgpu_box_interpolate: bad argument");
  for (int d = 0; d < 3; ++d)
    if (n[d] < 1 || !(hi[d] > lo[d])) return set_error(GLGPU_ERR_ARG, "glgpu_box_interpolate: invalid box");
  const int64_t sx = 1, sy = n[0] + 1, sz = static_cast<int64_t>(n[0] + 1) * (n[1] + 1);
  for (int64_t p = 0; p < n_points; ++p)
    {
      int64_t i0[3];
      double t[3];
      for (int d = 0; d < 3; ++d)
        {
          const double u = (xyz[3 * p + d] - lo[d]) / (hi[d] - lo[d]) * n[d];
          int64_t c = static_cast<int64_t>(std::floor(u));
          c = std::min<int64_t>(std::max<int64_t>(c, 0), n[d] - 1);
          i0[d] = c;
          t[d] = std::min(1.0, std::max(0.0, u - static_cast<double>(c)));
        }
      double *out = x + 18 * p;
      for (int c = 0; c < 18; ++c) out[c] = 0.0;
      for (int v = 0; v < 8; ++v)
        {
          double w = 1.0;
          int64_t node = 0;
          const int64_t st[3] = {sx, sy, sz};
          for (int d = 0; d < 3; ++d)
            {
              const int b = (v >> d) & 1;
              w *= b ? t[d] : 1.0 - t[d];
              node += (i0[d] + b) * st[d];
            }
          if (w == 0.0) continue;
          for (int c = 0; c < 18; ++c) out[c] += w * x_box[18 * node + c];
        }
    }
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_bphase_guess(double p, double t, int scc, int n_nodes, double noise_sigma,
                                           uint64_t seed, double *x)
{
  if (!x || n_nodes < 0) return set_error(GLGPU_ERR_ARG, "glgpu_bphase_guess: bad argument");
  double mp[13];
  if (matep_eval(p, t, scc != 0, mp) != 0) return set_error(GLGPU_ERR_ARG, "glgpu_bphase_guess: bad (p, t)");
  // setup_uniform_B-phase.cc:248: gap_B * 0.577350269f (single-precision literal)
  const double diag = mp[7] * static_cast<double>(0.577350269f);
  for (int64_t i = 0; i < static_cast<int64_t>(n_nodes); ++i)
    for (int c = 0; c < 18; ++c)
      {
        double v = (c == 0 || c == 4 || c == 8) ? diag : 0.0;
        if (noise_sigma > 0) v += noise_sigma * gaussian(seed, static_cast<uint64_t>(18 * i + c));
        x[18 * i + c] = v;
      }
  return GLGPU_OK;
}
