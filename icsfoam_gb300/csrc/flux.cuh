// Per-face inviscid flux functions (device).
//
// Each follows the field-expression order of the reference so the FP64
// result tracks the oracle to round-off:
//   AUSM+up : ausmPlusUpFluxScheme.C:73-299 (Liou 2006, beta = 1/8,
//             alpha = 3/16, Kp = 0.25 pressure diffusion with the 0.2 sign
//             guard, Ku = 0.25 velocity diffusion when lowMachAusm)
//   HLLC    : hllcFluxScheme.C:70-240 (Roe-averaged wave speeds, pos()/neg()
//             switches with x >= 0 -> 1)
//   Roe     : roeFluxScheme.C:41-409 (P |Lambda| P^-1 dissipation with the
//             Harten entropy fix)
// um is the MRF face velocity (frame velocity . n, zero outside MRF zones):
// it makes the normal velocities relative and adds the pressure work where
// each scheme adds it (ausmPlusUpFluxScheme.C:101-102,293; hllcFluxScheme.C:
// 157-161,217-218; roeFluxScheme.C:362-363,406-408).
#pragma once

#include "dual.cuh"
#include "ics_internal.cuh"

namespace ics {

// ------------------------------------------------ phase-lag cyclic neighbours
// The neighbour value of instance J across a phase-lag cyclic face is
// sum_K P_JK f_K(partner cell of instance K) for the fields the reference
// phase-lags (phaseLagCyclicFvPatchField::patchNeighbourField: rho, p, the U
// components, E, H and the sound speed); the others keep the plain cyclic
// neighbour of their own instance.
__device__ __forceinline__ int plag_mode(const DevMesh& m, int b) {
  return m.plagMode ? m.plagMode[m.bpatch[b]] : 0;
}
template <typename Real, typename Fn>
__device__ __forceinline__ Real plag_sum(const DevMesh& m, int b, int pc, Fn f) {
  const int n = m.nInst, J = pc / m.Nc, cl = pc - J * m.Nc;
  const double* P = m.plagP + ((size_t)m.bpatch[b] * n + J) * n;
  Real s = Real(0.0);
  for (int K = 0; K < n; ++K) s = s + P[K] * f(K * m.Nc + cl);
  return s;
}
// the velocity from its component arrays: combined as it is (mode 1) or
// combined and rotated into this side's frame (mode 2, cylindrical coordinates)
template <typename Real>
__device__ __forceinline__ void plag_vec(const DevMesh& m, int b, int pc, const Real* Ux, const Real* Uy,
                                         const Real* Uz, Real v[3]) {
  Real a[3];
  a[0] = plag_sum<Real>(m, b, pc, [&](int c) { return Ux[c]; });
  a[1] = plag_sum<Real>(m, b, pc, [&](int c) { return Uy[c]; });
  a[2] = plag_sum<Real>(m, b, pc, [&](int c) { return Uz[c]; });
  if (plag_mode(m, b) == 2) {
    const double* R = m.patches[m.bpatch[b]].R;
    for (int k = 0; k < 3; ++k) v[k] = R[3 * k] * a[0] + R[3 * k + 1] * a[1] + R[3 * k + 2] * a[2];
  } else {
    for (int k = 0; k < 3; ++k) v[k] = a[k];
  }
}
// field k of the q layout [NQ][N]; the sound speed's neighbour is
// sqrt(gamma/psi) of the instances (for AUSM+up's c* as well, as the reference)
template <typename Real>
__device__ __forceinline__ Real plag_q(const DevMesh& m, const Real* q, int k, int b, int pc) {
  const int N = m.N;
  if (k == Q_UX || k == Q_UY || k == Q_UZ) {
    Real v[3];
    plag_vec<Real>(m, b, pc, q + Q_UX * N, q + Q_UY * N, q + Q_UZ * N, v);
    return v[k - Q_UX];
  }
  if (k == Q_C) {
    const double g = m.gamma;
    return plag_sum<Real>(m, b, pc, [&](int c) { return sqrt(g * (q[Q_P * N + c] / q[Q_RHO * N + c])); });
  }
  if (k == Q_H)
    return plag_sum<Real>(m, b, pc, [&](int c) { return q[Q_E * N + c] + q[Q_P * N + c] / q[Q_RHO * N + c]; });
  return plag_sum<Real>(m, b, pc, [&](int c) { return q[k * N + c]; });
}

// Face state; Real = double for the residual, Dual for its tangent
template <typename Real>
struct FStateT {
  Real rho, p, U[3], E, H, c;
};
using FState = FStateT<double>;

template <typename Real>
__device__ __forceinline__ Real sq(const Real& x) {
  return x * x;
}
template <typename A, typename B>
__device__ __forceinline__ auto dot3(const A* a, const B* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <typename Real>
__device__ __forceinline__ double pos0d(const Real& s) {
  return val(s) >= 0 ? 1.0 : 0.0;
}
template <typename Real>
__device__ __forceinline__ double negd(const Real& s) {
  return val(s) < 0 ? 1.0 : 0.0;
}

// out: phi, phiUx, phiUy, phiUz, phiE
template <typename Real>
__device__ __forceinline__ void flux_ausm(const FStateT<Real>& L, const FStateT<Real>& R, const double S[3],
                                          double magS, int lowMach, double um, Real out[5]) {
  const Real unL = dot3(L.U, S) / magS - um;
  const Real unR = dot3(R.U, S) / magS - um;
  const Real cl = sq(L.c) / fmax(L.c, unL);
  const Real cr = sq(R.c) / fmax(R.c, -unR);
  const Real cf = fmin(cl, cr);
  const Real ML = unL / cf;
  Real Mplus, pplus;
  if (fabs(ML) < 1.0) {
    const Real ML2p = 0.25 * sq(ML + 1);
    const Real ML2m = -0.25 * sq(ML - 1);
    Mplus = ML2p * (1 - 2 * ML2m);
    pplus = ML2p * (2 - ML - 3 * ML * ML2m);
  } else {
    Mplus = fmax(ML, 0.0);
    pplus = ML > 0 ? 1.0 : 0.0;
  }
  const Real MR = unR / cf;
  Real Mminus, pminus;
  if (fabs(MR) < 1.0) {
    const Real MR2m = -0.25 * sq(MR - 1);
    const Real MR2p = 0.25 * sq(MR + 1);
    Mminus = MR2m * (1 + 2 * MR2p);
    pminus = MR2m * (-2 - MR + 3 * MR * MR2p);
  } else {
    Mminus = fmin(MR, 0.0);
    pminus = MR < 0 ? 1.0 : 0.0;
  }
  Real M12 = Mplus + Mminus;
  Real p12 = pplus * L.p + pminus * R.p;
  const Real Mmean = 0.5 * (sq(unL) + sq(unR)) / sq(cf);
  const Real MDiff = -0.25 * fmax((1.0 - Mmean), 0.0) * (R.p - L.p) / (0.5 * (L.rho + R.rho) * sq(cf));
  if ((M12 > 0.0 && M12 + MDiff <= 0.0) || (M12 < 0.0 && M12 + MDiff >= 0.0))
    M12 += 0.2 * MDiff;
  else
    M12 += MDiff;
  if (lowMach) p12 += -0.25 * pplus * pminus * (L.rho + R.rho) * cf * (unR - unL);
  const bool left = M12 >= 0;
  const FStateT<Real>& up = left ? L : R;
  const Real rhoa = M12 * cf * up.rho;
  out[0] = rhoa * magS;
  out[1] = rhoa * up.U[0] * magS + p12 * S[0];
  out[2] = rhoa * up.U[1] * magS + p12 * S[1];
  out[3] = rhoa * up.U[2] * magS + p12 * S[2];
  out[4] = rhoa * up.H * magS + p12 * um * magS;
}

template <typename Real>
__device__ __forceinline__ void flux_hllc(const FStateT<Real>& L, const FStateT<Real>& R, const double n[3],
                                          double magS, double gInterp, double um, Real out[5]) {
  const Real coefR = sqrt(fmax(VSMALL, R.rho) / fmax(VSMALL, L.rho));
  const Real icr = 1.0 / (coefR + 1.0);  // one FP64 reciprocal for the four Roe averages
  Real uAvg[3];
  for (int k = 0; k < 3; ++k) uAvg[k] = (coefR * R.U[k] + L.U[k]) * icr;
  const Real HAvg = (coefR * R.H + L.H) * icr;
  const Real cAvg = sqrt(fabs((gInterp - 1.0) * (HAvg - 0.5 * dot3(uAvg, uAvg))));
  const Real uMag_l = dot3(L.U, n) - um;
  const Real uMag_r = dot3(R.U, n) - um;
  const Real uMagAvg = dot3(uAvg, n) - um;
  const Real Sl = fmin(uMag_l - L.c, uMagAvg - cAvg);
  const Real Sr = fmax(uMag_r + R.c, uMagAvg + cAvg);
  const Real rl = L.rho, rr = R.rho, pl = L.p, pr = R.p;
  const Real Sm = (rr * uMag_r * (Sr - uMag_r) - rl * uMag_l * (Sl - uMag_l) + pl - pr) /
                    (rr * (Sr - uMag_r) - rl * (Sl - uMag_l));
  const double coefSl = pos0d(Sl);
  const double coefSr = negd(Sr);
  const double coefSm = pos0d(Sm);
  const double coefSlm = (1.0 - coefSl) * coefSm;
  const double coefSmr = (1.0 - coefSm) * (1.0 - coefSr);
  if ((coefSl != 0.0) + (coefSlm != 0.0) + (coefSmr != 0.0) + (coefSr != 0.0) == 1) {
    // The usual case: exactly one wave region has a non-zero switch, and the
    // switched sum below reduces to that region's flux (x + 0 = x, 1 x = x),
    // so only that flux is evaluated: the plain flux of one side (Sl >= 0 or
    // Sr < 0) or one side's star flux.  The two states are selected, not
    // blended, so this costs no FP64 work.
    const bool left = coefSl != 0.0 || coefSlm != 0.0;
    const FStateT<Real>& X = left ? L : R;
    const Real uX = left ? uMag_l : uMag_r;
    if (coefSl != 0.0 || coefSr != 0.0) {
      out[0] = X.rho * uX * magS;
      for (int k = 0; k < 3; ++k) out[1 + k] = (X.rho * uX * X.U[k] + X.p * n[k]) * magS;
      out[4] = X.rho * X.H * uX * magS;
      return;
    }
    const Real SX = left ? Sl : Sr;
    const Real iX = 1.0 / (SX - Sm);
    out[0] = Sm * iX * ((SX - uX) * X.rho) * magS;
    const Real pStar = X.rho * (uX - SX) * (uX - Sm) + X.p;
    for (int k = 0; k < 3; ++k) {
      const Real rus = iX * ((SX - uX) * X.rho * X.U[k] + (pStar - X.p) * n[k]);
      out[1 + k] = (Sm * rus + pStar * n[k]) * magS;
    }
    const Real rhoEStar = iX * ((SX - uX) * (X.rho * X.E) - X.p * uX + pStar * Sm);
    out[4] = (Sm * (rhoEStar + pStar) + pStar * um) * magS;
    return;
  }
  // one reciprocal per wave pair, shared by the mass, momentum and energy star fluxes
  const Real il = 1.0 / (Sl - Sm), ir = 1.0 / (Sr - Sm);
  const Real fluxRhoStar_l = Sm * il * ((Sl - uMag_l) * rl);
  const Real fluxRhoStar_r = Sm * ir * ((Sr - uMag_r) * rr);
  out[0] = (coefSl * rl * uMag_l + coefSlm * fluxRhoStar_l + coefSmr * fluxRhoStar_r + coefSr * rr * uMag_r) * magS;
  const Real pStar_l = rl * (uMag_l - Sl) * (uMag_l - Sm) + pl;
  const Real pStar_r = rr * (uMag_r - Sr) * (uMag_r - Sm) + pr;
  for (int k = 0; k < 3; ++k) {
    const Real rusl = il * ((Sl - uMag_l) * rl * L.U[k] + (pStar_l - pl) * n[k]);
    const Real rusr = ir * ((Sr - uMag_r) * rr * R.U[k] + (pStar_r - pr) * n[k]);
    const Real fl = Sm * rusl + pStar_l * n[k];
    const Real fr = Sm * rusr + pStar_r * n[k];
    out[1 + k] = (coefSl * (rl * uMag_l * L.U[k] + pl * n[k]) + coefSlm * fl + coefSmr * fr +
                  coefSr * (rr * uMag_r * R.U[k] + pr * n[k])) *
                 magS;
  }
  const Real rhoEStar_l = il * ((Sl - uMag_l) * (rl * L.E) - pl * uMag_l + pStar_l * Sm);
  const Real rhoEStar_r = ir * ((Sr - uMag_r) * (rr * R.E) - pr * uMag_r + pStar_r * Sm);
  const Real fEl = Sm * (rhoEStar_l + pStar_l) + pStar_l * um;
  const Real fEr = Sm * (rhoEStar_r + pStar_r) + pStar_r * um;
  out[4] = (coefSl * rl * L.H * uMag_l + coefSlm * fEl + coefSmr * fEr + coefSr * rr * R.H * uMag_r) * magS;
}

template <typename A, typename B, typename C>
__device__ __forceinline__ void cross3(const A* a, const B* b, C* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

template <typename Real>
__device__ __forceinline__ void flux_roe(const FStateT<Real>& L, const FStateT<Real>& R, const double n[3],
                                         double magS, double gI, double eps, double um, Real out[5]) {
  const Real coefR = sqrt(fmax(VSMALL, R.rho) / fmax(VSMALL, L.rho));
  const Real rD = coefR * L.rho;
  Real rU[3];
  const Real icr = 1.0 / (coefR + 1.0);
  for (int k = 0; k < 3; ++k) rU[k] = (coefR * R.U[k] + L.U[k]) * icr;
  const Real rH = (coefR * R.H + L.H) * icr;
  const Real rC = sqrt(fabs((gI - 1.0) * (rH - 0.5 * dot3(rU, rU))));
  const Real uMag_l = dot3(L.U, n), uMag_r = dot3(R.U, n);
  const Real uProj = dot3(rU, n) - um;
  const double a1 = gI - 1;
  const Real theta = 0.5 * a1 * dot3(rU, rU);
  const Real c2 = sq(rC);
  const Real a2 = 1 / (rD * rC * sqrt(2.0));
  const Real a3 = rD / (rC * sqrt(2.0));
  const Real a4 = (theta + c2) / a1;
  const Real a5 = 1 - theta / c2;
  const Real a6 = theta / a1;
  Real cUn[3];
  cross3(rU, n, cUn);
  Real invP11[3], invP13[3], invP22[3], invP32[3];
  Real invP12[3][3];
  for (int i = 0; i < 3; ++i) {
    invP11[i] = (n[i] * a5) - cUn[i] / rD;
    invP13[i] = -a1 / c2 * n[i];
    invP22[i] = -a2 * (a1 * rU[i] - rC * n[i]);
    invP32[i] = -a2 * (a1 * rU[i] + rC * n[i]);
    for (int j = 0; j < 3; ++j) invP12[i][j] = (a1 / c2 * n[i]) * rU[j];
  }
  invP12[0][1] += n[2] / rD;
  invP12[0][2] -= n[1] / rD;
  invP12[1][0] -= n[2] / rD;
  invP12[1][2] += n[0] / rD;
  invP12[2][0] += n[1] / rD;
  invP12[2][1] -= n[0] / rD;
  const Real invP21 = a2 * (theta - rC * uProj);
  const Real invP23 = a1 * a2;
  const Real invP31 = a2 * (theta + rC * uProj);
  const Real invP33 = a1 * a2;
  Real L1 = fabs(uProj), L2 = fabs(uProj + rC), L3 = fabs(uProj - rC);
  const Real epsilon = eps * fmax(L2, L3);
  if (L1 < epsilon) L1 = (sq(L1) + sq(epsilon)) / (2.0 * epsilon);
  if (L2 < epsilon) L2 = (sq(L2) + sq(epsilon)) / (2.0 * epsilon);
  if (L3 < epsilon) L3 = (sq(L3) + sq(epsilon)) / (2.0 * epsilon);
  Real P21[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P21[i][j] = rU[i] * n[j];
  P21[0][1] -= n[2] * rD;
  P21[0][2] += n[1] * rD;
  P21[1][0] += n[2] * rD;
  P21[1][2] -= n[0] * rD;
  P21[2][0] -= n[1] * rD;
  P21[2][1] += n[0] * rD;
  Real P22[3], P23[3], P31[3];
  for (int i = 0; i < 3; ++i) {
    P22[i] = a3 * (rU[i] + rC * n[i]);
    P23[i] = a3 * (rU[i] - rC * n[i]);
    P31[i] = n[i] * a6 + rD * cUn[i];
  }
  const Real P12 = a3, P13 = a3;
  const Real P32 = a3 * (a4 + rC * uProj);
  const Real P33 = a3 * (a4 - rC * uProj);
  // differences of conservative states
  const Real dRho = R.rho - L.rho;
  Real dRhoU[3];
  for (int k = 0; k < 3; ++k) dRhoU[k] = R.rho * R.U[k] - L.rho * L.U[k];
  const Real dRhoE = R.rho * R.E - L.rho * L.E;
  // continuity row
  Real P11L[3] = {n[0] * L1, n[1] * L1, n[2] * L1};
  const Real dCR = dot3(P11L, invP11) + (L2 * P12 * invP21) + (L3 * P13 * invP31);
  Real dCU[3];
  for (int j = 0; j < 3; ++j)
    dCU[j] = (P11L[0] * invP12[0][j] + P11L[1] * invP12[1][j] + P11L[2] * invP12[2][j]) + (L2 * P12 * invP22[j]) +
             (L3 * P13 * invP32[j]);
  const Real dCE = dot3(P11L, invP13) + (L2 * P12 * invP23) + (L3 * P13 * invP33);
  Real ph = -0.5 * magS * (dCR * dRho + dot3(dCU, dRhoU) + dCE * dRhoE);
  // momentum rows
  Real pU[3];
  for (int i = 0; i < 3; ++i) {
    Real Pl[3] = {P21[i][0] * L1, P21[i][1] * L1, P21[i][2] * L1};
    const Real dMR = (Pl[0] * invP11[0] + Pl[1] * invP11[1] + Pl[2] * invP11[2]) + (L2 * invP21 * P22[i]) +
                       (L3 * invP31 * P23[i]);
    const Real dME = (Pl[0] * invP13[0] + Pl[1] * invP13[1] + Pl[2] * invP13[2]) + (L2 * invP23 * P22[i]) +
                       (L3 * invP33 * P23[i]);
    Real dMUdot = 0;
    for (int j = 0; j < 3; ++j) {
      const Real dMU = (Pl[0] * invP12[0][j] + Pl[1] * invP12[1][j] + Pl[2] * invP12[2][j]) +
                         (L2 * P22[i] * invP22[j]) + (L3 * P23[i] * invP32[j]);
      dMUdot += dMU * dRhoU[j];
    }
    pU[i] = -0.5 * magS * (dMR * dRho + dMUdot + dME * dRhoE);
  }
  Real P31L[3] = {P31[0] * L1, P31[1] * L1, P31[2] * L1};
  const Real dER = dot3(P31L, invP11) + (L2 * P32 * invP21) + (L3 * P33 * invP31);
  Real dEU[3];
  for (int j = 0; j < 3; ++j)
    dEU[j] = (P31L[0] * invP12[0][j] + P31L[1] * invP12[1][j] + P31L[2] * invP12[2][j]) + (L2 * P32 * invP22[j]) +
             (L3 * P33 * invP32[j]);
  const Real dEE = dot3(P31L, invP13) + (L2 * P32 * invP23) + (L3 * P33 * invP33);
  Real pE = -0.5 * magS * (dER * dRho + dot3(dEU, dRhoU) + dEE * dRhoE);
  const Real rn_l = L.rho * uMag_l, rn_r = R.rho * uMag_r;
  ph += 0.5 * magS * (rn_l + rn_r);
  for (int k = 0; k < 3; ++k) pU[k] += 0.5 * magS * (rn_l * L.U[k] + rn_r * R.U[k] + n[k] * (L.p + R.p));
  pE += 0.5 * magS * (rn_l * L.H + rn_r * R.H);
  if (um != 0.0) {  // the frame's share of the central flux (roeFluxScheme.C:406-408)
    const double hm = 0.5 * magS * um;
    ph -= hm * (L.rho + R.rho);
    for (int k = 0; k < 3; ++k) pU[k] -= hm * (L.rho * L.U[k] + R.rho * R.U[k]);
    pE -= hm * (L.rho * L.E + R.rho * R.E);
  }
  out[0] = ph;
  out[1] = pU[0];
  out[2] = pU[1];
  out[3] = pU[2];
  out[4] = pE;
}

}  // namespace ics
