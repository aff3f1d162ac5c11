// femgl_gb300: host driver for the GPU Newton path, a stand-in for the reference's
// sol/src/main.cc + FemGL<3>::run (femgl/src/run.cc:110-258) on two of its scenarios (the
// reference picks make_grid / setup_system by linking one source of each, here --scenario):
//   cube      femgl/src/makegrid_cube-z-normal_AdGR.cc + setup_uniform_B-phase.cc
//   pdw-slab  femgl/src/makegrid_retangle-z-AdGR_xy-periodic.cc +
//             setup_weak-coupling-PDW-configuration.cc: the rectangle of half lengths "half x /
//             y / z length of retangle", 2^r cells per axis, x and y faces periodic, z faces
//             pair-breaking, and the PDW start of amplitude "amplitude u parameter" across the
//             slab (pdw_config.h:111-298), without noise.
//
// It reads the reference's configuration file format (deal.II ParameterHandler text:
// "subsection <name>", "set <key> = <value>", "end", '#' comments) with the keys and
// defaults of confreader/src/declare.cc:115-290, builds the 2^r x 2^r x 2^r cube of side
// 2 * "cube half side length" (pair-breaking z faces) or the periodic slab, evaluates the
// material parameters at (p, t), starts from the uniform B phase (setup_uniform_B-phase.cc:
// 238-263, plus optional seeded Gaussian noise) or the PDW state, and runs the Newton loop
// through the C ABI of
// include/glgpu.h: assemble_system, solve(tol of the cycle), newton_iteration, stop at
// |R| <= "converge accuracy".  Refinement cycles follow run.cc:156-256: a cycle ends when
// its residual stalls (change below "Cycle c refinement threshold") or converges; the next
// cycle refines globally ("Cycle c do global refinement") or adaptively (GPU Kelly
// estimate, the "adaptive refinment ratio" of cells with the largest estimates refined
// once, refine.cc:131-176) and transfers the solution.  The host mesher supports one
// adaptive level on top of any number of global ones; a further adaptive cycle ends the
// cycle loop with a note.  On the periodic slab a cell flagged next to a periodic face also
// flags its image cell across the box (the mesher refines both faces of a periodic pair
// alike), so a few more cells than the fixed number may be refined.
//
// usage: femgl_gb300 [configuration.prm] [--scenario cube|pdw-slab]
//                    [--precision mixed|fp64] [--precond mg|bj|cheb|none]
//                    [--noise sigma] [--seed s] [--out solution.bin] [--dry-run]
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "glgpu.h"

namespace
{
// "subsection/key" -> value, seeded with the reference's declared defaults
struct Config
{
  std::map<std::string, std::string> kv;

  Config()
  {
    const char *phys = "physical parameters/";
    const char *ctrl = "control parameters/";
    const std::pair<std::string, std::string> defaults[] = {
      {std::string(phys) + "pressure in bar", "0.0"},
      {std::string(phys) + "t_reduced", "0.0"},
      {std::string(phys) + "AdGR diffuse length", "1.0e10"},
      {std::string(phys) + "gaussian random mean value", "2.0"},
      {std::string(phys) + "gaussian random STD", "0.1"},
      {std::string(phys) + "trun on Strong Coupling Correction", "true"},
      {std::string(phys) + "amplitude u parameter", "1.0"},
      {std::string(ctrl) + "cube half side length", "20"},
      {std::string(ctrl) + "half x length of retangle", "20"},
      {std::string(ctrl) + "half y length of retangle", "20"},
      {std::string(ctrl) + "half z length of retangle", "20"},
      {std::string(ctrl) + "Number of refinements", "4"},
      {std::string(ctrl) + "Number of interations", "40"},
      {std::string(ctrl) + "Cycle 0 refinement threshold", "1.0e0"},
      {std::string(ctrl) + "Cycle 0 linear solver tol", "1.0e-1"},
      {std::string(ctrl) + "Cycle 1 refinement threshold", "1.0e0"},
      {std::string(ctrl) + "Cycle 1 do global refinement", "false"},
      {std::string(ctrl) + "Cycle 1 linear solver tol", "1.0e-1"},
      {std::string(ctrl) + "Cycle 2 refinement threshold", "1.0e0"},
      {std::string(ctrl) + "Cycle 2 do global refinement", "false"},
      {std::string(ctrl) + "Cycle 2 linear solver tol", "1.0e-1"},
      {std::string(ctrl) + "Cycle 3 refinement threshold", "1.0e0"},
      {std::string(ctrl) + "Cycle 3 do global refinement", "false"},
      {std::string(ctrl) + "Cycle 3 linear solver tol", "1.0e-1"},
      {std::string(ctrl) + "Cycle 4 do global refinement", "false"},
      {std::string(ctrl) + "Cycle 4 linear solver tol", "1.0e-1"},
      {std::string(ctrl) + "adaptive refinment ratio", "0.3"},
      {std::string(ctrl) + "adaptive coarsen ratio", "0.0"},
      {std::string(ctrl) + "converge accuracy", "5.0e-6"},
      {std::string(ctrl) + "Number of initial global refinments", "4"},
      {std::string(ctrl) + "maximum linear iteration number", "10000"},
      {std::string(ctrl) + "Using dampped Newton iteration", "true"},
      {std::string(ctrl) + "primary step length of dampped newton iteration", "0.83"},
    };
    for (const auto &d : defaults) kv[d.first] = d.second;
  }

  static std::string trim(const std::string &s)
  {
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
  }

  bool read(const std::string &path, std::string &err)
  {
    std::ifstream in(path);
    if (!in)
      {
        err = "cannot open " + path;
        return false;
      }
    std::vector<std::string> stack;
    std::string line;
    int ln = 0;
    while (std::getline(in, line))
      {
        ++ln;
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        line = trim(line);
        if (line.empty()) continue;
        if (line.compare(0, 11, "subsection ") == 0)
          stack.push_back(trim(line.substr(11)));
        else if (line == "end")
          {
            if (stack.empty())
              {
                err = path + ":" + std::to_string(ln) + ": 'end' without subsection";
                return false;
              }
            stack.pop_back();
          }
        else if (line.compare(0, 4, "set ") == 0)
          {
            const size_t eq = line.find('=');
            if (eq == std::string::npos)
              {
                err = path + ":" + std::to_string(ln) + ": 'set' without '='";
                return false;
              }
            std::string key;
            for (const auto &s : stack) key += s + "/";
            key += trim(line.substr(4, eq - 4));
            kv[key] = trim(line.substr(eq + 1));
          }
        else
          {
            err = path + ":" + std::to_string(ln) + ": cannot parse '" + line + "'";
            return false;
          }
      }
    if (!stack.empty())
      {
        err = path + ": subsection '" + stack.back() + "' not closed";
        return false;
      }
    return true;
  }

  std::string get(const std::string &key) const
  {
    auto it = kv.find(key);
    return it == kv.end() ? std::string() : it->second;
  }
  double num(const std::string &key) const { return std::strtod(get(key).c_str(), nullptr); }
  bool flag(const std::string &key) const
  {
    const std::string v = get(key);
    return v == "true" || v == "1" || v == "yes";
  }
};

int fail(const char *what)
{
  std::fprintf(stderr, "femgl_gb300: %s: %s\n", what, glgpu_last_error());
  return 1;
}
} // namespace

int main(int argc, char **argv)
{
  std::string prm_path = "configuration.prm", out_path;
  int precision = GLGPU_MIXED, precond = GLGPU_PC_MULTIGRID;
  double noise = 0.0;
  uint64_t seed = 0;
  bool dry = false, pdw = false;
  for (int i = 1; i < argc; ++i)
    {
      const std::string a = argv[i];
      auto next = [&](const char *name) -> std::string {
        if (i + 1 >= argc)
          {
            std::fprintf(stderr, "femgl_gb300: %s needs a value\n", name);
            std::exit(2);
          }
        return argv[++i];
      };
      if (a == "--precision")
        {
          const std::string v = next("--precision");
          precision = (v == "fp64") ? GLGPU_FP64 : GLGPU_MIXED;
        }
      else if (a == "--precond")
        {
          const std::string v = next("--precond");
          precond = v == "bj" ? GLGPU_PC_BLOCK_JACOBI
                  : v == "cheb" ? GLGPU_PC_CHEBYSHEV
                  : v == "none" ? GLGPU_PC_NONE
                                : GLGPU_PC_MULTIGRID;
        }
      else if (a == "--scenario")
        {
          const std::string v = next("--scenario");
          if (v != "cube" && v != "pdw-slab")
            {
              std::fprintf(stderr, "femgl_gb300: unknown scenario %s (cube, pdw-slab)\n", v.c_str());
              return 2;
            }
          pdw = v == "pdw-slab";
        }
      else if (a == "--noise")
        noise = std::strtod(next("--noise").c_str(), nullptr);
      else if (a == "--seed")
        seed = std::strtoull(next("--seed").c_str(), nullptr, 10);
      else if (a == "--out")
        out_path = next("--out");
      else if (a == "--dry-run")
        dry = true;
      else if (!a.empty() && a[0] != '-')
        prm_path = a;
      else
        {
          std::fprintf(stderr, "femgl_gb300: unknown option %s\n", a.c_str());
          return 2;
        }
    }
  Config conf;
  std::string err;
  if (!conf.read(prm_path, err))
    {
      std::fprintf(stderr, "femgl_gb300: %s\n", err.c_str());
      return 2;
    }
  const std::string P = "physical parameters/", C = "control parameters/";
  const double p = conf.num(P + "pressure in bar"), t = conf.num(P + "t_reduced");
  const bool scc = conf.flag(P + "trun on Strong Coupling Correction");
  const double bt = conf.num(P + "AdGR diffuse length");
  const double half = conf.num(C + "cube half side length");
  const double half_r[3] = {conf.num(C + "half x length of retangle"), conf.num(C + "half y length of retangle"),
                            conf.num(C + "half z length of retangle")};
  const double amp_u = conf.num(P + "amplitude u parameter");
  const int nref = static_cast<int>(conf.num(C + "Number of initial global refinments"));
  const int n_iter = static_cast<int>(conf.num(C + "Number of interations"));
  const double tol0 = conf.num(C + "Cycle 0 linear solver tol");
  const double acc = conf.num(C + "converge accuracy");
  const int n_cycles = static_cast<int>(conf.num(C + "Number of refinements"));
  const double ratio = conf.num(C + "adaptive refinment ratio"), coarsen = conf.num(C + "adaptive coarsen ratio");
  int n = 1 << nref;
  if (pdw)
    std::printf("femgl_gb300: %s  p = %g bar, t = %g, SCC %s, periodic slab %g x %g x %g (x, y periodic), %d^3 "
                "cells, PDW start u = %g\n", glgpu_version(), p, t, scc ? "on" : "off", 2 * half_r[0], 2 * half_r[1],
                2 * half_r[2], n, amp_u);
  else
    std::printf("femgl_gb300: %s  p = %g bar, t = %g, SCC %s, cube half side %g, %d^3 cells\n", glgpu_version(), p,
                t, scc ? "on" : "off", half, n);
  for (int d = 0; d < 3 && pdw; ++d)
    if (!(half_r[d] > 0.0))
      {
        std::fprintf(stderr, "femgl_gb300: the half lengths of the rectangle must be > 0\n");
        return 2;
      }
  std::printf("  Newton: <= %d iterations, linear tol %g, converge accuracy %g, %s, %s\n", n_iter + 1, tol0, acc,
              precision == GLGPU_FP64 ? "FP64" : "mixed FP32/FP64",
              precond == GLGPU_PC_MULTIGRID ? "multigrid" : precond == GLGPU_PC_BLOCK_JACOBI ? "block-Jacobi"
                                            : precond == GLGPU_PC_CHEBYSHEV ? "Chebyshev" : "unpreconditioned");
  if (bt < 1e10) std::printf("  Robin (AdGR) term on the pair-breaking z faces, diffuse length %g\n", bt);
  if (!(bt > 0.0))
    {
      std::fprintf(stderr, "femgl_gb300: AdGR diffuse length must be > 0\n");
      return 2;
    }
  if (n_cycles > 4)
    {
      std::fprintf(stderr, "femgl_gb300: at most 4 refinement cycles (run.cc declares cycles 0-4)\n");
      return 2;
    }
  if (n_cycles > 0) std::printf("  refinement cycles: %d (adaptive ratio %g)\n", n_cycles, ratio);
  if (dry) return 0;

  // material parameters at (p, t)
  double mp[13];
  if (glgpu_matep(p, t, scc ? 1 : 0, mp)) return fail("matep");
  glgpu_params prm;
  glgpu_default_params(&prm);
  prm.alpha = mp[0];
  for (int k = 0; k < 5; ++k) prm.beta[k] = mp[1 + k];
  prm.precision = precision;
  prm.precond = precond;
  prm.gmres_max_iter = static_cast<int>(conf.num(C + "maximum linear iteration number"));
  prm.ls_step = conf.num(C + "primary step length of dampped newton iteration");
  prm.damped = conf.flag(C + "Using dampped Newton iteration") ? 1 : 0;
  prm.bt = bt;

  // cube, or the slab with periodic x / y faces; pair-breaking z faces (zero orbital-z column)
  // either way; cells of an adaptive level
  const double lo[3] = {pdw ? -half_r[0] : -half, pdw ? -half_r[1] : -half, pdw ? -half_r[2] : -half};
  const double hi[3] = {-lo[0], -lo[1], -lo[2]};
  const int dxy[2] = {pdw ? 2 : 0, pdw ? 2 : 0};
  struct Mesh
  {
    int nn = 0, nc = 0, nh = 0;
    std::vector<double> xyz, hw;
    std::vector<int32_t> cell, hptr, hpar;
    std::vector<uint32_t> mask;
  } M;
  auto make_mesh = [&](const int8_t *flags) -> bool {
    const int cells[3] = {n, n, n};
    auto call = [&](bool sizes) {
      return flags ? glgpu_mesh_box_refine(lo, hi, cells, flags, dxy, &M.nn, &M.nc, &M.nh,
                                           sizes ? nullptr : M.xyz.data(), sizes ? nullptr : M.cell.data(),
                                           sizes ? nullptr : M.mask.data(), sizes ? nullptr : M.hptr.data(),
                                           sizes ? nullptr : M.hpar.data(), sizes ? nullptr : M.hw.data())
                   : glgpu_mesh_box(lo, hi, cells, 0.0, dxy, &M.nn, &M.nc, &M.nh, sizes ? nullptr : M.xyz.data(),
                                    sizes ? nullptr : M.cell.data(), sizes ? nullptr : M.mask.data(),
                                    sizes ? nullptr : M.hptr.data(), sizes ? nullptr : M.hpar.data(),
                                    sizes ? nullptr : M.hw.data());
    };
    if (call(true)) return false;
    M.xyz.resize(3 * static_cast<size_t>(M.nn));
    M.cell.resize(8 * static_cast<size_t>(M.nc));
    M.mask.resize(M.nn);
    M.hptr.resize(static_cast<size_t>(M.nn) + 1);
    M.hpar.resize(M.nh > 0 ? M.nh : 1);
    M.hw.resize(M.nh > 0 ? M.nh : 1);
    return call(false) == GLGPU_OK;
  };
  if (!make_mesh(nullptr)) return fail("mesh");
  glgpu_ctx *ctx = nullptr;
  auto open = [&]() -> bool {
    glgpu_mesh mesh{3, M.nn, M.nc, M.xyz.data(), M.cell.data(), M.mask.data(), M.hptr.data(), M.hpar.data(),
                    M.hw.data()};
    if (ctx) glgpu_destroy(ctx);
    ctx = nullptr;
    return glgpu_create(&mesh, &prm, 1, &ctx) == GLGPU_OK;
  };
  if (!open()) return fail("create");
  std::vector<double> x(18 * static_cast<size_t>(M.nn));
  const glgpu_status st0 = pdw ? glgpu_pdw_guess(p, t, scc ? 1 : 0, amp_u, half_r[2], M.nn, M.xyz.data(), x.data())
                               : glgpu_bphase_guess(p, t, scc ? 1 : 0, M.nn, noise, seed, x.data());
  if (st0 != GLGPU_OK || glgpu_set_solution(ctx, x.data())) return fail("initial state");

  const char *thr_key[4] = {"Cycle 0 refinement threshold", "Cycle 1 refinement threshold",
                            "Cycle 2 refinement threshold", "Cycle 3 refinement threshold"};
  const char *tol_key[5] = {"Cycle 0 linear solver tol", "Cycle 1 linear solver tol", "Cycle 2 linear solver tol",
                            "Cycle 3 linear solver tol", "Cycle 4 linear solver tol"};
  const char *glob_key[4] = {"Cycle 1 do global refinement", "Cycle 2 do global refinement",
                             "Cycle 3 do global refinement", "Cycle 4 do global refinement"};
  bool adaptive_done = false, converged = false;
  double res = 0.0, gpu_ms = 0.0;
  int total_newton = 0, total_its = 0;
  for (int cycle = 0; cycle <= n_cycles; ++cycle)
    {
      if (cycle > 0)
        {
          // refine_grid (refine.cc:110-176): global or adaptive, then solution transfer
          const bool global = conf.flag(C + glob_key[cycle - 1]);
          if (!global && adaptive_done)
            {
              std::printf("  note: cycle %d would refine an adaptively refined mesh a second level; the host mesher "
                          "supports one adaptive level, so the cycles end here\n", cycle);
              break;
            }
          if (global && adaptive_done)
            {
              std::printf("  note: cycle %d would refine an adaptively refined mesh globally; the cycles end here\n",
                          cycle);
              break;
            }
          std::vector<double> xu(x.size());
          if (glgpu_get_solution(ctx, xu.data())) return fail("get_solution");
          const int n_old = n;
          std::vector<int8_t> flags;
          if (global)
            {
              n *= 2;
              if (!make_mesh(nullptr)) return fail("mesh");
            }
          else
            {
              flags.resize(M.nc);
              if (glgpu_estimate_error(ctx, nullptr) || glgpu_refine_flags(ctx, ratio, coarsen, flags.data()))
                return fail("error estimate");
              // mirror the flags of the cells on periodic faces (cells x fastest), to a fixed point
              for (bool changed = pdw; changed;)
                {
                  changed = false;
                  auto mark = [&](int i, int j, int k) {
                    int8_t &f = flags[(static_cast<size_t>(k) * n + j) * n + i];
                    if (f <= 0)
                      {
                        f = 1;
                        changed = true;
                      }
                  };
                  for (int k = 0; k < n; ++k)
                    for (int j = 0; j < n; ++j)
                      for (int i = 0; i < n; ++i)
                        {
                          if (flags[(static_cast<size_t>(k) * n + j) * n + i] <= 0) continue;
                          if (i == 0 || i == n - 1) mark(n - 1 - i, j, k);
                          if (j == 0 || j == n - 1) mark(i, n - 1 - j, k);
                        }
                }
              if (!make_mesh(flags.data())) return fail("mesh");
              adaptive_done = true;
            }
          const int cells_old[3] = {n_old, n_old, n_old};
          x.assign(18 * static_cast<size_t>(M.nn), 0.0);
          if (glgpu_box_interpolate(lo, hi, cells_old, xu.data(), M.nn, M.xyz.data(), x.data()))
            return fail("solution transfer");
          if (!open()) return fail("create");
          if (glgpu_set_solution(ctx, x.data())) return fail("set_solution");
          std::printf("refinement cycle %d (%s): %d cells, %d nodes, %d hanging-constraint entries\n", cycle,
                      global ? "global" : "adaptive", M.nc, M.nn, M.nh);
        }
      const double tol = conf.num(C + tol_key[cycle]);
      const double thr = cycle < 4 ? conf.num(C + thr_key[cycle]) : 0.0;
      double last = 0.0;
      glgpu_event_start(ctx);
      for (int it = 0; it <= n_iter; ++it)
        {
          double rhs = 0.0, r = 0.0;
          int its = 0, trials = 0;
          if (glgpu_assemble_system(ctx, &rhs)) return fail("assemble_system");
          const glgpu_status st = glgpu_solve(ctx, tol, &its);
          if (st != GLGPU_OK && st != GLGPU_ERR_NOT_CONVERGED) return fail("solve");
          if (glgpu_newton_iteration(ctx, &r, &trials)) return fail("newton_iteration");
          total_its += its;
          ++total_newton;
          res = r;
          std::printf("  iteration %2d: |rhs| %.6e, GMRES %4d%s, line-search trials %d, |R| %.6e\n", it, rhs, its,
                      st == GLGPU_ERR_NOT_CONVERGED ? " (limit)" : "", trials, r);
          if (std::fabs(r - last) < thr && r > acc && cycle < n_cycles) break; // stalled: refine
          if (r <= acc) break;
          last = r;
        }
      double ms = 0.0;
      glgpu_event_stop(ctx, &ms);
      gpu_ms += ms;
      if (res <= acc)
        {
          converged = true;
          break;
        }
    }
  double F = 0.0;
  if (glgpu_free_energy(ctx, &F)) return fail("free_energy");
  std::printf("%s after %d Newton iterations (%d GMRES): |R| = %.6e, F = %.15e, %.1f ms on the GPU\n",
              converged ? "converged" : "NOT converged", total_newton, total_its, res, F, gpu_ms);
  if (!out_path.empty())
    {
      x.resize(18 * static_cast<size_t>(M.nn));
      if (glgpu_get_solution(ctx, x.data())) return fail("get_solution");
      FILE *f = std::fopen(out_path.c_str(), "wb");
      if (!f || std::fwrite(x.data(), sizeof(double), x.size(), f) != x.size())
        {
          std::fprintf(stderr, "femgl_gb300: cannot write %s\n", out_path.c_str());
          if (f) std::fclose(f);
          return 1;
        }
      std::fclose(f);
    }
  glgpu_destroy(ctx);
  return converged ? 0 : 1;
}
