// Viscous terms of the residual and the LF viscous Jacobian coefficient.
//
//   visc_cell  (cell gather)  Gauss linear gradients of U (tensor, dU_j/dx_i)
//                             and e, laminar mu (constant or Sutherland),
//                             alphaEff = (Cp/Cv) mu/Pr, tauMC = mu dev2(T(grad U))
//   visc_face  (internal face) laplacian(mu, U) and laplacian(alphaEff, e)
//                             with the non-orthogonal correction of
//                             "Gauss linear corrected", div(tauMC) and
//                             div(sigmaDotU . S) face terms, and
//                             sf2 = 0.5 (mu+alpha)/rho |S| deltaCoeffs
//   visc_bface (boundary face) the same with boundary values; the boundary
//                             gradient has its normal part replaced by the
//                             patch snGrad (psi_b - psi_P) deltaCoeffs_b
// Reference: residualsUpdate.H:16-43 (terms kept separate, each divided by V),
// viscousFluxScheme.C:234-247 (LaxFriedrichJacobian).
#include <type_traits>

#include "flux.cuh"
#include "ics_internal.cuh"

namespace ics {

struct ViscParams {
  double R, Cv, Cp, gamma, mu, Pr, As, Ts;
  int sutherland;
};

template <typename Real>
__device__ __forceinline__ Real mu_of(const ViscParams& P, const Real& T) {
  return P.sutherland ? P.As * sqrt(T) / (1.0 + P.Ts / T) : Real(P.mu);
}
template <typename Real>
__device__ __forceinline__ Real alpha_of(const ViscParams& P, const Real& mu) {
  return P.Cp / P.Cv * (mu / P.Pr);
}

// vc layout [24][N]: 0-8 grad U (3i+j), 9-11 grad e, 12-20 tau (3i+j), 21 mu, 22 alpha, 23 e

template <typename Real = double>
__global__ void __launch_bounds__(128) k_visc_cell(DevMesh m, ViscParams P, const Real* __restrict__ W,
                                                   const Real* __restrict__ prim, const double* __restrict__ TB,
                                                   const double* __restrict__ UB, Real* __restrict__ vc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int N = m.N, F = m.F, B = m.B;
  Real Uc[3] = {prim[2 * N + c], prim[3 * N + c], prim[4 * N + c]};
  const Real ec = W[5 * c + 4] / W[5 * c] - 0.5 * dot3(Uc, Uc);
  Real g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, ge[3] = {0, 0, 0};
  for (int e = m.cptr[c]; e < m.cptr[c + 1]; ++e) {
    const int code = m.cface[e];
    const bool isOwn = code >= 0;
    const int f = isOwn ? code : ~code;
    const int other = isOwn ? m.nei[f] : m.own[f];
    const double wf = m.w[f];
    const double S[3] = {m.Sf[f], m.Sf[F + f], m.Sf[2 * F + f]};
    const Real Uo[3] = {prim[2 * N + other], prim[3 * N + other], prim[4 * N + other]};
    const Real eo = W[5 * other + 4] / W[5 * other] - 0.5 * dot3(Uo, Uo);
    for (int j = 0; j < 3; ++j) {
      const Real a = isOwn ? Uc[j] : Uo[j], b = isOwn ? Uo[j] : Uc[j];
      const Real sf = wf * (a - b) + b;
      for (int i = 0; i < 3; ++i) g[3 * i + j] = isOwn ? g[3 * i + j] + S[i] * sf : g[3 * i + j] - S[i] * sf;
    }
    const Real a = isOwn ? ec : eo, b = isOwn ? eo : ec;
    const Real sf = wf * (a - b) + b;
    for (int i = 0; i < 3; ++i) ge[i] = isOwn ? ge[i] + S[i] * sf : ge[i] - S[i] * sf;
  }
  for (int e = m.bptr[c]; e < m.bptr[c + 1]; ++e) {
    const int b = m.bface[e];
    const double S[3] = {m.bSf[b], m.bSf[B + b], m.bSf[2 * B + b]};
    const int pc = m.bpartner ? m.bpartner[b] : -1;
    if (pc >= 0) {
      // coupled face: interpolate with the partner, its velocity rotated
      const double* Rm = m.patches[m.bpatch[b]].R;
      const double wb = m.bw[b];
      const Real Un[3] = {prim[2 * N + pc], prim[3 * N + pc], prim[4 * N + pc]};
      const Real en = W[5 * pc + 4] / W[5 * pc] - 0.5 * dot3(Un, Un);
      Real upv[3];
      if (plag_mode(m, b))  // U phase-lagged across an HB phase-lag patch
        plag_vec(m, b, pc, prim + 2 * N, prim + 3 * N, prim + 4 * N, upv);
      else
        for (int j = 0; j < 3; ++j) upv[j] = Rm[3 * j] * Un[0] + Rm[3 * j + 1] * Un[1] + Rm[3 * j + 2] * Un[2];
      for (int j = 0; j < 3; ++j) {
        const Real up = upv[j];
        const Real sf = wb * (Uc[j] - up) + up;
        for (int i = 0; i < 3; ++i) g[3 * i + j] += S[i] * sf;
      }
      const Real sf = wb * (ec - en) + en;
      for (int i = 0; i < 3; ++i) ge[i] += S[i] * sf;
      continue;
    }
    const double Ub[3] = {UB[b], UB[B + b], UB[2 * B + b]};
    const double eb = P.Cv * TB[b];
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) g[3 * i + j] += S[i] * Ub[j];
    for (int i = 0; i < 3; ++i) ge[i] += S[i] * eb;
  }
  const double Vc = m.V[c];
  for (int q = 0; q < 9; ++q) g[q] /= Vc;
  for (int q = 0; q < 3; ++q) ge[q] /= Vc;
  const Real mu = mu_of(P, prim[N + c]);
  const Real tr = g[0] + g[4] + g[8];
  for (int q = 0; q < 9; ++q) vc[q * N + c] = g[q];
  for (int q = 0; q < 3; ++q) vc[(9 + q) * N + c] = ge[q];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) vc[(12 + 3 * i + j) * N + c] = mu * (g[3 * j + i] - (i == j ? (2.0 / 3.0) * tr : Real(0.0)));
  vc[21 * N + c] = mu;
  vc[22 * N + c] = alpha_of(P, mu);
  vc[23 * N + c] = ec;
}

// fv layout [8][F+B]: lapU(3), divTau(3), divSig, lapE
template <typename Real = double>
__global__ void __launch_bounds__(128) k_visc_face(DevMesh m, const Real* __restrict__ vc,
                                                   const Real* __restrict__ W, const Real* __restrict__ prim,
                                                   Real* __restrict__ fv, double* __restrict__ sf2,
                                                   double* __restrict__ vj, int FB) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.F) return;
  const int N = m.N, F = m.F;
  const int o = m.own[f], n = m.nei[f];
  const double wf = m.w[f];
  auto lin = [&](int q) { return wf * (vc[q * N + o] - vc[q * N + n]) + vc[q * N + n]; };
  const Real muf = lin(21), alf = lin(22);
  const double ms = m.magSf[f];
  const double S[3] = {m.Sf[f], m.Sf[F + f], m.Sf[2 * F + f]};
  const double nodc = m.nodc[f];
  double k[3];
  for (int i = 0; i < 3; ++i) k[i] = m.nf[i * F + f] - m.dCC[i * F + f] * nodc;
  Real gUf[9], tf[9];
  for (int q = 0; q < 9; ++q) {
    gUf[q] = lin(q);
    tf[q] = lin(12 + q);
  }
  Real Uf[3], snU[3];
  for (int j = 0; j < 3; ++j) {
    const Real a = prim[(2 + j) * N + o], b = prim[(2 + j) * N + n];
    Uf[j] = wf * (a - b) + b;
    const Real corr = k[0] * gUf[j] + k[1] * gUf[3 + j] + k[2] * gUf[6 + j];
    snU[j] = nodc * (b - a) + corr;
  }
  const Real ml = muf * ms;
  for (int j = 0; j < 3; ++j) fv[j * FB + f] = ml * snU[j];
  for (int j = 0; j < 3; ++j) fv[(3 + j) * FB + f] = S[0] * tf[j] + S[1] * tf[3 + j] + S[2] * tf[6 + j];
  Real sig[3];
  for (int i = 0; i < 3; ++i) {
    Real s = 0;
    for (int j = 0; j < 3; ++j) s += (muf * gUf[3 * i + j] + tf[3 * i + j]) * Uf[j];
    sig[i] = s;
  }
  fv[6 * FB + f] = dot3(sig, S);
  const Real gef[3] = {lin(9), lin(10), lin(11)};
  const Real snE = nodc * (vc[23 * N + n] - vc[23 * N + o]) + dot3(k, gef);
  fv[7 * FB + f] = (alf * ms) * snE;
  if constexpr (std::is_same<Real, double>::value) {  // Jacobian coefficient: not part of the tangent
    const double rhof = wf * (W[5 * o] - W[5 * n]) + W[5 * n];
    const double lamv = (muf + alf) / rhof;
    sf2[f] = 0.5 * lamv * ms * m.dc[f];
    if (vj) {  // laplacian coefficients of the non-LF Jacobian (blockFvOperatorsTemplates.C:398-399)
      vj[f] = muf * ms * m.dc[f];
      vj[FB + f] = alf * ms * m.dc[f];
    }
  }
}

template <typename Real = double>
__global__ void k_visc_bface(DevMesh m, ViscParams P, const Real* __restrict__ vc, const Real* __restrict__ prim,
                             const double* __restrict__ TB, const double* __restrict__ UBv, Real* __restrict__ fv,
                             double* __restrict__ vj, int FB) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m.B) return;
  if (m.bpartner && m.bpartner[b] >= 0) return;  // cyclic faces: k_visc_cface
  const int N = m.N, B = m.B, F = m.F;
  const int o = m.bcell[b];
  const double ms = m.bmagSf[b];
  const double S[3] = {m.bSf[b], m.bSf[B + b], m.bSf[2 * B + b]};
  const double n[3] = {S[0] / ms, S[1] / ms, S[2] / ms};
  const double UB[3] = {UBv[b], UBv[B + b], UBv[2 * B + b]};
  const double muB = mu_of(P, TB[b]);
  const double alB = alpha_of(P, muB);
  const double eB = P.Cv * TB[b];
  const double dcb = m.bdc[b];
  Real snU[3];
  for (int j = 0; j < 3; ++j) snU[j] = (UB[j] - prim[(2 + j) * N + o]) * dcb;
  const Real snE = (eB - vc[23 * N + o]) * dcb;
  Real g[9];
  for (int q = 0; q < 9; ++q) g[q] = vc[q * N + o];
  for (int j = 0; j < 3; ++j) {
    const Real ng = n[0] * vc[j * N + o] + n[1] * vc[(3 + j) * N + o] + n[2] * vc[(6 + j) * N + o];
    for (int i = 0; i < 3; ++i) g[3 * i + j] += n[i] * (snU[j] - ng);
  }
  const Real tr = g[0] + g[4] + g[8];
  Real tb[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) tb[3 * i + j] = muB * (g[3 * j + i] - (i == j ? (2.0 / 3.0) * tr : Real(0.0)));
  const double ml = muB * ms;
  for (int j = 0; j < 3; ++j) fv[j * FB + F + b] = ml * snU[j];
  for (int j = 0; j < 3; ++j) fv[(3 + j) * FB + F + b] = S[0] * tb[j] + S[1] * tb[3 + j] + S[2] * tb[6 + j];
  Real sig[3];
  for (int i = 0; i < 3; ++i) {
    Real s = 0;
    for (int j = 0; j < 3; ++j) s += (muB * g[3 * i + j] + tb[3 * i + j]) * UB[j];
    sig[i] = s;
  }
  fv[6 * FB + F + b] = dot3(sig, S);
  fv[7 * FB + F + b] = (alB * ms) * snE;
  if (vj) {  // patch mu and alphaEff for the non-LF boundary terms (viscousFluxScheme.C:57-58)
    vj[F + b] = muB;
    vj[FB + F + b] = alB;
  }
}

// Cyclic faces: the internal-face terms with the partner's vectors rotated
// (R v) and its tensors rotated (R t R^T) into this side's frame, the
// partner-side centre at C + delta (coupled snGrad and its non-orthogonal
// correction), plus the LF coefficient of the coupled laplacian.
template <typename Real = double>
__global__ void __launch_bounds__(128) k_visc_cface(DevMesh m, const Real* __restrict__ vc,
                                                    const Real* __restrict__ W, const Real* __restrict__ prim,
                                                    Real* __restrict__ fv, double* __restrict__ sf2,
                                                    double* __restrict__ vj, int FB) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (i0 >= m.ncyc) return;
  const int N = m.N, F = m.F, B = m.B;
  const int b = m.cyc_face[i0];
  const int o = m.bcell[b], pc = m.bpartner[b];
  const double* Rm = m.patches[m.bpatch[b]].R;
  const double wf = m.bw[b];
  auto lin = [&](const Real& a, const Real& bb) { return wf * (a - bb) + bb; };
  const Real muf = lin(vc[21 * N + o], vc[21 * N + pc]), alf = lin(vc[22 * N + o], vc[22 * N + pc]);
  const double ms = m.bmagSf[b];
  const double S[3] = {m.bSf[b], m.bSf[B + b], m.bSf[2 * B + b]};
  const double nodc = m.bnodc[b];
  double k[3];
  for (int i = 0; i < 3; ++i) k[i] = m.bnf[i * B + b] - m.bdelta[i * B + b] * nodc;
  Real gUf[9], tf[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      Real sg = 0, st = 0;
      for (int kk = 0; kk < 3; ++kk)
        for (int l = 0; l < 3; ++l) {
          sg += Rm[3 * i + kk] * vc[(3 * kk + l) * N + pc] * Rm[3 * j + l];
          st += Rm[3 * i + kk] * vc[(12 + 3 * kk + l) * N + pc] * Rm[3 * j + l];
        }
      gUf[3 * i + j] = lin(vc[(3 * i + j) * N + o], sg);
      tf[3 * i + j] = lin(vc[(12 + 3 * i + j) * N + o], st);
    }
  const Real Un[3] = {prim[2 * N + pc], prim[3 * N + pc], prim[4 * N + pc]};
  Real upv[3];
  if (plag_mode(m, b))
    plag_vec(m, b, pc, prim + 2 * N, prim + 3 * N, prim + 4 * N, upv);
  else
    for (int j = 0; j < 3; ++j) upv[j] = Rm[3 * j] * Un[0] + Rm[3 * j + 1] * Un[1] + Rm[3 * j + 2] * Un[2];
  Real Uf[3], snU[3];
  for (int j = 0; j < 3; ++j) {
    const Real up = upv[j];
    const Real uo = prim[(2 + j) * N + o];
    Uf[j] = lin(uo, up);
    const Real corr = k[0] * gUf[j] + k[1] * gUf[3 + j] + k[2] * gUf[6 + j];
    snU[j] = nodc * (up - uo) + corr;
  }
  const Real ml = muf * ms;
  for (int j = 0; j < 3; ++j) fv[j * FB + F + b] = ml * snU[j];
  for (int j = 0; j < 3; ++j) fv[(3 + j) * FB + F + b] = S[0] * tf[j] + S[1] * tf[3 + j] + S[2] * tf[6 + j];
  Real sig[3];
  for (int i = 0; i < 3; ++i) {
    Real s = 0;
    for (int j = 0; j < 3; ++j) s += (muf * gUf[3 * i + j] + tf[3 * i + j]) * Uf[j];
    sig[i] = s;
  }
  fv[6 * FB + F + b] = dot3(sig, S);
  Real gef[3];
  for (int i = 0; i < 3; ++i) {
    const Real gp = Rm[3 * i] * vc[9 * N + pc] + Rm[3 * i + 1] * vc[10 * N + pc] + Rm[3 * i + 2] * vc[11 * N + pc];
    gef[i] = lin(vc[(9 + i) * N + o], gp);
  }
  const Real snE = nodc * (vc[23 * N + pc] - vc[23 * N + o]) + dot3(k, gef);
  fv[7 * FB + F + b] = (alf * ms) * snE;
  if constexpr (std::is_same<Real, double>::value) {
    const double rhof = lin(W[5 * o], W[5 * pc]);
    sf2[F + b] = 0.5 * ((muf + alf) / rhof) * ms * m.bdc[b];
    if (vj) {
      vj[F + b] = muf * ms * m.bdc[b];
      vj[FB + F + b] = alf * ms * m.bdc[b];
    }
  }
}

void launch_viscous(Handle& h) {
  if (!h.cfg.c.viscous) return;
  ViscParams P;
  P.R = h.cfg.c.R;
  P.Cv = h.cfg.Cv;
  P.Cp = h.cfg.c.Cp;
  P.gamma = h.cfg.gamma;
  P.mu = h.cfg.c.mu;
  P.Pr = h.cfg.c.Pr;
  P.As = h.cfg.c.As;
  P.Ts = h.cfg.c.Ts;
  P.sutherland = h.cfg.c.sutherland;
  const int FB = h.m.F + h.m.B;
  double* vj = h.vjac;  // written in both Jacobian modes: the mode may change between residual and assembly
  ICS_LAUNCH(h, ICS_K_VISC, k_visc_cell<<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m, P, h.W, h.prim, h.TB, h.UB,
                                                                                     h.vcell));
  if (h.m.F)
    ICS_LAUNCH(h, ICS_K_VISC, k_visc_face<<<grid_for(h.m.F, 128), 128, 0, h.stream>>>(h.m, h.vcell, h.W, h.prim,
                                                                                       h.fvisc, h.vsf2, vj, FB));
  if (h.m.B)
    ICS_LAUNCH(h, ICS_K_VISC, k_visc_bface<<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, P, h.vcell, h.prim, h.TB,
                                                                                        h.UB, h.fvisc, vj, FB));
  if (h.m.ncyc)
    ICS_LAUNCH(h, ICS_K_VISC, k_visc_cface<<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(h.m, h.vcell, h.W, h.prim,
                                                                                           h.fvisc, h.vsf2, vj, FB));
  ICS_CUDA(cudaGetLastError());
}

// tangent of the viscous face terms for the tangent state (W, prim) in tW, tprim
void launch_viscous_tangent(Handle& h, const Dual* W, const Dual* prim, Dual* vc, Dual* fv) {
  ViscParams P;
  P.R = h.cfg.c.R;
  P.Cv = h.cfg.Cv;
  P.Cp = h.cfg.c.Cp;
  P.gamma = h.cfg.gamma;
  P.mu = h.cfg.c.mu;
  P.Pr = h.cfg.c.Pr;
  P.As = h.cfg.c.As;
  P.Ts = h.cfg.c.Ts;
  P.sutherland = h.cfg.c.sutherland;
  const int FB = h.m.F + h.m.B;
  ICS_LAUNCH(h, ICS_K_TANGENT, k_visc_cell<Dual><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m, P, W, prim, h.TB,
                                                                                             h.UB, vc));
  if (h.m.F)
    ICS_LAUNCH(h, ICS_K_TANGENT, k_visc_face<Dual><<<grid_for(h.m.F, 128), 128, 0, h.stream>>>(h.m, vc, W, prim, fv,
                                                                                               nullptr, nullptr, FB));
  if (h.m.B)
    ICS_LAUNCH(h, ICS_K_TANGENT, k_visc_bface<Dual><<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, P, vc, prim, h.TB,
                                                                                                h.UB, fv, nullptr, FB));
  if (h.m.ncyc)
    ICS_LAUNCH(h, ICS_K_TANGENT, k_visc_cface<Dual><<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(h.m, vc, W, prim, fv,
                                                                                                   nullptr, nullptr, FB));
  ICS_CUDA(cudaGetLastError());
}

}  // namespace ics
