// State update and boundary conditions.
//
//   update  (cell)          W += dW, rho/e bounding, T = e/Cv, p = rho/psi,
//                           re-derived rhoU and rhoE (updateFields.H:7-78)
//   bc      (boundary face) p, then U, then T boundary values from the
//                           interior and the previous boundary values; psi on
//                           the patch comes from the previous boundary T, as
//                           in thermo.correct() before the correction
//                           (updateFields.H:80-104)
//   bound   (cell gather)   pseudo Courant reduction around cells whose
//                           density or energy fell under the lower bound
//                           (boundLocalTimeStep.H:1-97)
// Patch kinds restate OpenFOAM's zeroGradient, slip, fixedValue,
// totalPressure, totalTemperature and pressureInletOutletVelocity.
#include "flux.cuh"
#include "ics_internal.cuh"

namespace ics {

__global__ void k_update(int N, double* __restrict__ W, const double* __restrict__ dW, double* __restrict__ prim,
                         double R, double Cv, double rhoMin, double eMin, double eMax, int useTMax,
                         int* __restrict__ bounded) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double rho = W[5 * i] + dW[5 * i];
  double rU[3] = {W[5 * i + 1] + dW[5 * i + 1], W[5 * i + 2] + dW[5 * i + 2], W[5 * i + 3] + dW[5 * i + 3]};
  double rE = W[5 * i + 4] + dW[5 * i + 4];
  rho = fmax(rho, rhoMin);
  double U[3] = {rU[0] / rho, rU[1] / rho, rU[2] / rho};
  double e = rE / rho - 0.5 * dot3(U, U);
  int nb = 0;
  if (e < eMin) {
    e = eMin;
    nb = 1;
  }
  if (useTMax && e > eMax) {
    e = eMax;
    nb = 1;
  }
  if (nb) atomicAdd(bounded, 1);
  const double T = e / Cv;
  const double p = rho / (1.0 / (R * T));
  W[5 * i] = rho;
  W[5 * i + 1] = rho * U[0];
  W[5 * i + 2] = rho * U[1];
  W[5 * i + 3] = rho * U[2];
  W[5 * i + 4] = rho * (e + 0.5 * dot3(U, U));
  prim[i] = p;
  prim[N + i] = T;
  prim[2 * N + i] = U[0];
  prim[3 * N + i] = U[1];
  prim[4 * N + i] = U[2];
}

__global__ void k_bc(DevMesh m, const double* __restrict__ prim, double* __restrict__ pB, double* __restrict__ TB,
                     double* __restrict__ UB, const double* __restrict__ phiB, double R, double gamma, double TMin,
                     double TMax, int useTMax) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m.B) return;
  const int B = m.B, N = m.N;
  const Patch pt = m.patches[m.bpatch[b]];
  const int ci = m.bcell[b];
  if (m.bpartner && m.bpartner[b] >= 0) {
    // coupled patch: weighted mean of this side's cell and the partner's,
    // the partner's velocity rotated into this side's frame
    // (coupledFvPatchField::evaluate with cyclic patchNeighbourField)
    const int pc = m.bpartner[b];
    const double wb = m.bw[b];
    const double* Rm = pt.R;
    // phase-lag cyclic (HB): p and U of the instances combined, T plain
    const bool plag = plag_mode(m, b) != 0;
    const double pn = plag ? plag_sum<double>(m, b, pc, [&](int c) { return prim[c]; }) : prim[pc];
    pB[b] = wb * (prim[ci] - pn) + pn;
    double upv[3];
    if (plag) {
      plag_vec(m, b, pc, prim + 2 * N, prim + 3 * N, prim + 4 * N, upv);
    } else {
      const double Un[3] = {prim[2 * N + pc], prim[3 * N + pc], prim[4 * N + pc]};
      for (int k = 0; k < 3; ++k) upv[k] = Rm[3 * k] * Un[0] + Rm[3 * k + 1] * Un[1] + Rm[3 * k + 2] * Un[2];
    }
    for (int k = 0; k < 3; ++k) {
      const double up = upv[k];
      UB[k * B + b] = wb * (prim[(2 + k) * N + ci] - up) + up;
    }
    double T = wb * (prim[N + ci] - prim[N + pc]) + prim[N + pc];
    T = fmax(T, TMin);
    if (useTMax) T = fmax(T, TMax);
    TB[b] = T;
    return;
  }
  const double psiB = 1.0 / (R * TB[b]);
  const double gM1ByG = (gamma - 1.0) / gamma;
  const double Uc[3] = {prim[2 * N + ci], prim[3 * N + ci], prim[4 * N + ci]};
  double Uold[3] = {UB[b], UB[B + b], UB[2 * B + b]};
  const double phi = phiB[b];
  // p
  double p = pB[b];
  switch (pt.kind) {
    case ICS_PATCH_ZERO_GRADIENT:
    case ICS_PATCH_SLIP:
    case ICS_PATCH_ISOTHERMAL_WALL: p = prim[ci]; break;
    case ICS_PATCH_FIXED:
    case ICS_PATCH_PRESSURE_OUTLET: p = pt.p; break;
    case ICS_PATCH_TOTAL_INLET:
      p = pt.p0 / pow((1.0 + 0.5 * psiB * gM1ByG * (1.0 - pos0d(phi)) * dot3(Uold, Uold)), 1.0 / gM1ByG);
      break;
    default: break;
  }
  // U
  double U[3] = {Uold[0], Uold[1], Uold[2]};
  const double n[3] = {m.bnf[b], m.bnf[B + b], m.bnf[2 * B + b]};
  switch (pt.kind) {
    case ICS_PATCH_ZERO_GRADIENT:
    case ICS_PATCH_PRESSURE_OUTLET:
      for (int k = 0; k < 3; ++k) U[k] = Uc[k];
      break;
    case ICS_PATCH_SLIP: {
      const double un = dot3(n, Uc);
      for (int k = 0; k < 3; ++k) U[k] = Uc[k] - n[k] * un;
      break;
    }
    case ICS_PATCH_FIXED:
      for (int k = 0; k < 3; ++k) U[k] = pt.U[k];
      break;
    case ICS_PATCH_ISOTHERMAL_WALL: U[0] = U[1] = U[2] = 0.0; break;
    case ICS_PATCH_TOTAL_INLET: {
      const double vf = negd(phi);
      for (int i = 0; i < 3; ++i) {
        double s = 0;
        for (int j = 0; j < 3; ++j) {
          const double Iij = (i == j ? 1.0 : 0.0);
          const double vfij = vf * (Iij - n[i] * n[j]);
          s += (Iij - vfij) * Uc[j];
        }
        U[i] = 0.0 + s;
      }
      break;
    }
    default: break;
  }
  // MRF: fixed-value patches keep the frame velocity that
  // correctBoundaryVelocity assigned them; in the every-update mode every
  // included face is re-assigned before T is evaluated (HB updateFields.H:86-88)
  if (m.mrfBIn && m.mrfBIn[b] &&
      (m.mrfEvery || pt.kind == ICS_PATCH_FIXED || pt.kind == ICS_PATCH_ISOTHERMAL_WALL))
    for (int k = 0; k < 3; ++k) U[k] = m.mrfBU[k * B + b];
  // T
  double T = TB[b];
  switch (pt.kind) {
    case ICS_PATCH_ZERO_GRADIENT:
    case ICS_PATCH_SLIP:
    case ICS_PATCH_PRESSURE_OUTLET: T = prim[N + ci]; break;
    case ICS_PATCH_FIXED:
    case ICS_PATCH_ISOTHERMAL_WALL: T = pt.T; break;
    case ICS_PATCH_TOTAL_INLET: T = pt.T0 / (1.0 + 0.5 * psiB * gM1ByG * (1.0 - pos0d(phi)) * dot3(U, U)); break;
    default: break;
  }
  T = fmax(T, TMin);
  if (useTMax) T = fmax(T, TMax);  // updateFields.H:86-89 as written
  pB[b] = p;
  TB[b] = T;
  UB[b] = U[0];
  UB[B + b] = U[1];
  UB[2 * B + b] = U[2];
}

// primitive initial state: W and prim from (p, U[N][3], T) staged in prim
__global__ void k_set_primitive(int N, double R, double Cv, const double* __restrict__ pin,
                                const double* __restrict__ Uin, const double* __restrict__ Tin, double* __restrict__ W,
                                double* __restrict__ prim) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double p = pin[i], T = Tin[i];
  const double U[3] = {Uin[3 * i], Uin[3 * i + 1], Uin[3 * i + 2]};
  const double e = Cv * T;
  const double rho = (1.0 / (R * T)) * p;
  W[5 * i] = rho;
  W[5 * i + 1] = rho * U[0];
  W[5 * i + 2] = rho * U[1];
  W[5 * i + 3] = rho * U[2];
  W[5 * i + 4] = rho * (e + 0.5 * dot3(U, U));
  prim[i] = p;
  prim[N + i] = T;
  prim[2 * N + i] = U[0];
  prim[3 * N + i] = U[1];
  prim[4 * N + i] = U[2];
}

// boundary initial guess: interior values and the matching boundary mass flux
__global__ void k_bc_init(DevMesh m, const double* __restrict__ prim, double R, double* __restrict__ pB,
                          double* __restrict__ TB, double* __restrict__ UB, double* __restrict__ phiB) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m.B) return;
  const int B = m.B, N = m.N, ci = m.bcell[b];
  const double p = prim[ci], T = prim[N + ci];
  const double U[3] = {prim[2 * N + ci], prim[3 * N + ci], prim[4 * N + ci]};
  const double S[3] = {m.bSf[b], m.bSf[B + b], m.bSf[2 * B + b]};
  pB[b] = p;
  TB[b] = T;
  UB[b] = U[0];
  UB[B + b] = U[1];
  UB[2 * B + b] = U[2];
  phiB[b] = (1.0 / (R * T)) * p * dot3(U, S);
}

// primitives from W (set_conservative); Real = Dual for the tangent
template <typename Real>
__global__ void k_derive(int N, const Real* __restrict__ W, Real* __restrict__ prim, double R, double Cv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const Real rho = W[5 * i];
  const Real U[3] = {W[5 * i + 1] / rho, W[5 * i + 2] / rho, W[5 * i + 3] / rho};
  const Real e = W[5 * i + 4] / rho - 0.5 * dot3(U, U);
  const Real T = e / Cv;
  prim[i] = rho / (1.0 / (R * T));
  prim[N + i] = T;
  prim[2 * N + i] = U[0];
  prim[3 * N + i] = U[1];
  prim[4 * N + i] = U[2];
}

__global__ void k_bad(int N, const double* __restrict__ W, const double* __restrict__ Wprev, double lb,
                      int* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double rp = Wprev[5 * i], rEp = Wprev[5 * i + 4];
  const double up[3] = {Wprev[5 * i + 1] / rp, Wprev[5 * i + 2] / rp, Wprev[5 * i + 3] / rp};
  const double rhoMin = lb * rp;
  const double eMin = lb * (rEp / rp - 0.5 * dot3(up, up));
  const double r = W[5 * i];
  const double u[3] = {W[5 * i + 1] / r, W[5 * i + 2] / r, W[5 * i + 3] / r};
  const double eT = W[5 * i + 4] / r - 0.5 * dot3(u, u);
  bad[i] = (r < rhoMin || eT < eMin || eT < SMALL) ? 1 : 0;
}

__global__ void k_bound_factor(DevMesh m, const int* __restrict__ bad, double* __restrict__ pseudoCo) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  double f = 1.0;
  const bool self = bad[c] != 0;
  for (int e = m.cptr[c]; e < m.cptr[c + 1]; ++e) {
    const int code = m.cface[e];
    const int fc = code >= 0 ? code : ~code;
    const int other = code >= 0 ? m.nei[fc] : m.own[fc];
    if (self) f = fmin(0.5, f);
    if (bad[other]) f = fmin(0.75, f);
  }
  pseudoCo[c] *= f;
}

void launch_update(Handle& h, int* boundedDev) {
  const ics_config& c = h.cfg.c;
  const double eMin = h.cfg.Cv * c.T_min;
  const double eMax = h.cfg.Cv * c.T_max;
  const int useTMax = c.T_max < GREAT ? 1 : 0;
  ICS_LAUNCH(h, ICS_K_UPDATE, k_update<<<grid_for(h.m.N, 256), 256, 0, h.stream>>>(h.m.N, h.W, h.dW, h.prim, c.R, h.cfg.Cv, c.rho_min, eMin, eMax,
                                                        useTMax, boundedDev));
  ICS_CUDA(cudaGetLastError());
}

// MRFCoupledZone::correctBoundaryVelocity (MRFCoupledZone.C:594-619): the
// frame velocity on the included boundary faces
__global__ void k_mrf_bc(DevMesh m, double* __restrict__ UB) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m.B || !m.mrfBIn[b]) return;
  const int B = m.B;
  for (int k = 0; k < 3; ++k) UB[k * B + b] = m.mrfBU[k * B + b];
}

void launch_mrf_bc(Handle& h) {
  if (!h.m.B || !h.m.mrfBIn) return;
  ICS_LAUNCH(h, ICS_K_BC, k_mrf_bc<<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, h.UB));
  ICS_CUDA(cudaGetLastError());
}

void launch_bc(Handle& h) {
  if (!h.m.B) return;
  const ics_config& c = h.cfg.c;
  ICS_LAUNCH(h, ICS_K_BC, k_bc<<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, h.prim, h.pB, h.TB, h.UB, h.phiB, c.R, h.cfg.gamma, c.T_min,
                                                    c.T_max, c.T_max < GREAT ? 1 : 0));
  ICS_CUDA(cudaGetLastError());
}

void launch_set_primitive(Handle& h) {
  // staged inputs: scratch holds p (N), U (3N), T (N)
  const int N = h.m.N;
  ICS_LAUNCH(h, ICS_K_UPDATE, k_set_primitive<<<grid_for(N, 256), 256, 0, h.stream>>>(N, h.cfg.c.R, h.cfg.Cv, h.scratch, h.scratch + N,
                                                           h.scratch + 4 * N, h.W, h.prim));
  if (h.m.B)
    ICS_LAUNCH(h, ICS_K_BC, k_bc_init<<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, h.prim, h.cfg.c.R, h.pB, h.TB, h.UB, h.phiB));
  ICS_CUDA(cudaGetLastError());
  launch_bc(h);
}

void launch_derive_primitive(Handle& h) {
  ICS_LAUNCH(h, ICS_K_UPDATE, k_derive<<<grid_for(h.m.N, 256), 256, 0, h.stream>>>(h.m.N, h.W, h.prim, h.cfg.c.R, h.cfg.Cv));
  ICS_CUDA(cudaGetLastError());
}

void launch_derive_tangent(Handle& h, const Dual* W, Dual* prim) {
  ICS_LAUNCH(h, ICS_K_TANGENT, k_derive<Dual><<<grid_for(h.m.N, 256), 256, 0, h.stream>>>(h.m.N, W, prim, h.cfg.c.R,
                                                                                          h.cfg.Cv));
  ICS_CUDA(cudaGetLastError());
}

void launch_bound_local_timestep(Handle& h) {
  const ics_config& c = h.cfg.c;
  if (!c.local_timestepping || !c.local_timestepping_bounding) return;
  ICS_LAUNCH(h, ICS_K_BOUND, k_bad<<<grid_for(h.m.N, 256), 256, 0, h.stream>>>(h.m.N, h.W, h.Wprev, c.local_timestepping_lower_bound, h.ibuf));
  ICS_LAUNCH(h, ICS_K_BOUND, k_bound_factor<<<grid_for(h.m.N, 256), 256, 0, h.stream>>>(h.m, h.ibuf, h.pseudoCo));
  ICS_CUDA(cudaGetLastError());
}

}  // namespace ics
