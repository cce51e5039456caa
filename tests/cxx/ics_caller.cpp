// A C++ caller of the C ABI in include/icsfoam_gb300.h, the way a host solver
// (dbnsFoam's pseudo loop, outerLoop.H + updateFields.H) would drive it:
// describe a mesh, create a handle, set the initial fields, run pseudo
// iterations and read the state back.  Built twice by the tests:
//   * against the CUDA library (libicsgpu.so, the ics_ entry points), and
//   * with -DICS_CALLER_ORACLE against the oracle (libicsref.so), which
//     exports the same functions under the icsref_ prefix.
// Compiling it checks every declaration it uses against the header, and
// linking checks the library exports them, which a ctypes binding does not.
//
// The mesh is a channel of nx x ny x nz hex cells over [0,3]x[0,1]x[0,0.5]
// with a total-pressure inlet (x = 0), a static-pressure outlet (x = 3) and
// slip walls, in OpenFOAM's LDU order (owner < neighbour, faces sorted by
// owner then neighbour, boundary faces patch by patch).
//
// usage: ics_caller nx ny nz iterations precision(0|1)
// prints one line per iteration (rho L2 residual, GMRES cycles) and a final
// line with sum(W) per equation, all with 17 significant digits.
#ifdef ICS_CALLER_ORACLE
#define ics_default_config icsref_default_config
#define ics_create icsref_create
#define ics_destroy icsref_destroy
#define ics_last_error icsref_last_error
#define ics_set_primitive icsref_set_primitive
#define ics_pseudo_loop icsref_pseudo_loop
#define ics_pseudo_iteration icsref_pseudo_iteration
#define ics_get_state icsref_get_state
#endif
#include "icsfoam_gb300.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace {

struct Box {
  int nx, ny, nz;
  double Lx = 3.0, Ly = 1.0, Lz = 0.5;
  std::vector<int32_t> own, nei, bcell, bpatch;
  std::vector<double> Sf, Cf, w, dc, nodc, C, V, bSf, bCf, bdc;

  int id(int i, int j, int k) const { return i + nx * (j + ny * k); }

  Box(int nx_, int ny_, int nz_) : nx(nx_), ny(ny_), nz(nz_) {
    const double h[3] = {Lx / nx, Ly / ny, Lz / nz};
    const double area[3] = {h[1] * h[2], h[0] * h[2], h[0] * h[1]};
    const int n = nx * ny * nz;
    C.resize(3 * n);
    V.assign(n, h[0] * h[1] * h[2]);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const int c = id(i, j, k);
          C[3 * c] = (i + 0.5) * h[0];
          C[3 * c + 1] = (j + 0.5) * h[1];
          C[3 * c + 2] = (k + 0.5) * h[2];
        }
    // internal faces: for each cell its +x, +y, +z neighbours (ascending index)
    for (int c = 0; c < n; ++c) {
      const int i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
      const int nb[3] = {i + 1 < nx ? c + 1 : -1, j + 1 < ny ? c + nx : -1, k + 1 < nz ? c + nx * ny : -1};
      for (int d = 0; d < 3; ++d) {
        if (nb[d] < 0) continue;
        own.push_back(c);
        nei.push_back(nb[d]);
        for (int e = 0; e < 3; ++e) {
          Sf.push_back(e == d ? area[d] : 0.0);
          Cf.push_back(C[3 * c + e] + (e == d ? 0.5 * h[d] : 0.0));
        }
        w.push_back(0.5);
        dc.push_back(1.0 / h[d]);
        nodc.push_back(1.0 / h[d]);
      }
    }
    // boundary faces: patch 0 inlet (x-), 1 outlet (x+), 2 walls (y-, y+, z-, z+)
    auto bface = [&](int c, int d, double sign, int patch) {
      bcell.push_back(c);
      bpatch.push_back(patch);
      for (int e = 0; e < 3; ++e) {
        bSf.push_back(e == d ? sign * area[d] : 0.0);
        bCf.push_back(C[3 * c + e] + (e == d ? sign * 0.5 * h[d] : 0.0));
      }
      bdc.push_back(2.0 / h[d]);
    };
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j) bface(id(0, j, k), 0, -1.0, 0);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j) bface(id(nx - 1, j, k), 0, 1.0, 1);
    for (int k = 0; k < nz; ++k)
      for (int i = 0; i < nx; ++i) bface(id(i, 0, k), 1, -1.0, 2);
    for (int k = 0; k < nz; ++k)
      for (int i = 0; i < nx; ++i) bface(id(i, ny - 1, k), 1, 1.0, 2);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) bface(id(i, j, 0), 2, -1.0, 2);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) bface(id(i, j, nz - 1), 2, 1.0, 2);
  }
};

int fail(ics_handle h, const char* where, int st) {
  char msg[256] = "";
  if (h) ics_last_error(h, msg, sizeof(msg));
  std::fprintf(stderr, "%s failed with status %d: %s\n", where, st, msg);
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s nx ny nz iterations precision\n", argv[0]);
    return 2;
  }
  const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nz = std::atoi(argv[3]);
  const int iters = std::atoi(argv[4]), precision = std::atoi(argv[5]);
  Box box(nx, ny, nz);
  const double gamma = 1.4, R = 287.0, mach = 0.5, p0 = 1e5, T0 = 300.0;
  const double fac = 1.0 + 0.5 * (gamma - 1.0) * mach * mach;
  const double ps = p0 / std::pow(fac, gamma / (gamma - 1.0)), Ts = T0 / fac;

  ics_patch_desc patches[3] = {};
  patches[0].kind = ICS_PATCH_TOTAL_INLET;
  patches[0].p0 = p0;
  patches[0].T0 = T0;
  patches[1].kind = ICS_PATCH_PRESSURE_OUTLET;
  patches[1].p = ps;
  patches[2].kind = ICS_PATCH_SLIP;
  patches[2].is_wall = 1;

  ics_mesh_desc m = {};
  m.n_cells = nx * ny * nz;
  m.n_faces = (int32_t)box.own.size();
  m.n_bfaces = (int32_t)box.bcell.size();
  m.n_patches = 3;
  m.owner = box.own.data();
  m.neighbour = box.nei.data();
  m.Sf = box.Sf.data();
  m.Cf = box.Cf.data();
  m.weights = box.w.data();
  m.delta_coeffs = box.dc.data();
  m.nonorth_delta_coeffs = box.nodc.data();
  m.C = box.C.data();
  m.V = box.V.data();
  m.b_cell = box.bcell.data();
  m.b_patch = box.bpatch.data();
  m.b_Sf = box.bSf.data();
  m.b_Cf = box.bCf.data();
  m.b_delta_coeffs = box.bdc.data();
  m.patches = patches;
  m.solution_d[0] = m.solution_d[1] = m.solution_d[2] = 1;

  // fvSchemes / fvSolution of the case: HLLC, linearUpwind + cellLimited<
  // Venkatakrishnan>, GMRES(8) + LU-SGS, SER pseudo-CFL ramp 1 -> 100
  ics_config cfg;
  ics_default_config(&cfg);
  cfg.R = R;
  cfg.Cp = gamma * R / (gamma - 1.0);
  cfg.flux_scheme = ICS_FLUX_HLLC;
  cfg.recon_rho = cfg.recon_U = cfg.recon_T = ICS_RECON_MUSCL_VENKATAKRISHNAN;
  cfg.n_directions = 8;
  cfg.max_iter = 5;
  cfg.rel_tol = 1e-2;
  cfg.pseudo_co_num = 1.0;
  cfg.pseudo_co_num_max = 100.0;
  cfg.pseudo_tol = cfg.pseudo_tol_rel = 1e-30;
  cfg.precision = precision ? ICS_PREC_MIXED : ICS_PREC_FP64;

  ics_handle h = nullptr;
  int st = ics_create(&m, &cfg, &h);
  if (st) return fail(h, "ics_create", st);
  const int n = m.n_cells;
  std::vector<double> p(n), U(3 * n, 0.0), T(n, Ts);
  const double c = std::sqrt(gamma * R * Ts);
  for (int i = 0; i < n; ++i) {
    const double x = box.C[3 * i], y = box.C[3 * i + 1];
    p[i] = ps * (1.0 + 0.01 * std::sin(2.0 * x) * std::cos(3.0 * y));
    U[3 * i] = mach * c;
  }
  if ((st = ics_set_primitive(h, p.data(), U.data(), T.data()))) return fail(h, "ics_set_primitive", st);
  for (int it = 0; it < iters; ++it) {
    int32_t more = 0;
    if ((st = ics_pseudo_loop(h, &more))) return fail(h, "ics_pseudo_loop", st);
    ics_iter_stats s;
    if ((st = ics_pseudo_iteration(h, &s))) return fail(h, "ics_pseudo_iteration", st);
    std::printf("iter %d rho_l2 %.17g cycles %d\n", it, s.rho_l2_residual, s.perf.n_iterations);
  }
  std::vector<double> W(5 * (size_t)n);
  if ((st = ics_get_state(h, W.data(), nullptr, nullptr, nullptr))) return fail(h, "ics_get_state", st);
  double sum[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 5; ++k) sum[k] += W[5 * i + k];
  std::printf("sumW %.17g %.17g %.17g %.17g %.17g\n", sum[0], sum[1], sum[2], sum[3], sum[4]);
  ics_destroy(h);
  return 0;
}
