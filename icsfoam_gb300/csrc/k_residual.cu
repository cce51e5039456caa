// Residual pipeline: reconstructed fields -> gradients (+ limiter) ->
// face fluxes -> cell residual, local pseudo time step and ddtCoeff.
//
//   fields   (cell / boundary face)  q = rho, p, U, E, H, c          [NQ][N]
//   grad     (cell, face-ordered gather) Gauss linear gradient of each
//            reconstructed scalar; for MUSCL the cellLimited limiter is
//            fused in (it needs only the cell's own gradient and its
//            neighbours' values)                                       [NQ][3][N]
//   face     (internal face) left/right reconstruction + flux scheme,
//            linear-interpolated wave speed, reconstructed (U, E) kept
//            for the Jacobian                                          [5][F]
//   bface    (boundary face) L = R = boundary value
//   cellres  (cell, face-ordered gather) div of the fluxes, dual-time ddt,
//            source = R*V, SER update of the pseudo Courant number,
//            rPseudoDeltaT and ddtCoeff (setCoAndDeltaT.H)
//
// Reference: ausmPlusUpFluxScheme.C:73-299, hllcFluxScheme.C:70-240,
// roeFluxScheme.C:276-409, residualsUpdate.H:1-83, setCoAndDeltaT.H:39-141,
// dualTimeDdtScheme.C:111-126.  Reconstruction restates OpenFOAM's
// limitedScheme (NVD/TVD r with vanLeer or Minmod), linearUpwind and
// cellLimited<Venkatakrishnan|minmod> Gauss linear gradients.
#include <type_traits>

#include "residual.cuh"

namespace ics {

// ------------------------------------------------------------------ fields
// Real = double: cells and boundary faces; Real = Dual: the cells' tangents
// (boundary values are held fixed, their tangent is zero).
template <typename Real>
__global__ void k_fields(int N, int B, const Real* __restrict__ W, const Real* __restrict__ prim,
                         const double* __restrict__ pB, const double* __restrict__ TB,
                         const double* __restrict__ UB, ResParams P, Real* __restrict__ q,
                         double* __restrict__ bq, double* __restrict__ clin, double* __restrict__ bclin) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    const Real rho = W[5 * i];
    const Real p = prim[i], T = prim[N + i];
    const Real U0 = prim[2 * N + i], U1 = prim[3 * N + i], U2 = prim[4 * N + i];
    const Real E = P.Cv * T + 0.5 * (U0 * U0 + U1 * U1 + U2 * U2);
    const Real H = fmax(E, SMALL) + fmax(p / rho, SMALL);
    const Real psi = 1.0 / (P.R * T);
    const Real cl = sqrt(P.gamma / psi);
    q[Q_RHO * N + i] = rho;
    q[Q_P * N + i] = p;
    q[Q_UX * N + i] = U0;
    q[Q_UY * N + i] = U1;
    q[Q_UZ * N + i] = U2;
    q[Q_E * N + i] = E;
    q[Q_H * N + i] = H;
    q[Q_C * N + i] = P.scheme == ICS_FLUX_AUSMPLUSUP ? sqrt(P.cstarFac * H) : fmax(cl, VSMALL);
    if constexpr (is_fp64<Real>) clin[i] = cl;
  }
  if constexpr (is_fp64<Real>) {
    if (i < B) {
      const double p = pB[i], T = TB[i];
      const double U0 = UB[i], U1 = UB[B + i], U2 = UB[2 * B + i];
      const double psi = 1.0 / (P.R * T);
      const double rho = psi * p;
      const double E = P.Cv * T + 0.5 * (U0 * U0 + U1 * U1 + U2 * U2);
      const double H = fmax(E, SMALL) + fmax(p / rho, SMALL);
      const double cl = sqrt(P.gamma / psi);
      bq[Q_RHO * B + i] = rho;
      bq[Q_P * B + i] = p;
      bq[Q_UX * B + i] = U0;
      bq[Q_UY * B + i] = U1;
      bq[Q_UZ * B + i] = U2;
      bq[Q_E * B + i] = E;
      bq[Q_H * B + i] = H;
      bq[Q_C * B + i] = P.scheme == ICS_FLUX_AUSMPLUSUP ? sqrt(P.cstarFac * H) : fmax(cl, VSMALL);
      bclin[i] = cl;
    }
  }
}

// --------------------------------------------------------------- gradients
// One thread per cell; faces visited in increasing face index (the order the
// face-loop gradient accumulates them).  mask selects the fields, limited
// selects cellLimited (1 = minmod, 2 = Venkatakrishnan).
template <int LIMITED, typename Real = double>
__global__ void __launch_bounds__(128) k_grad(DevMesh m, const Real* __restrict__ q, const double* __restrict__ bq,
                                              unsigned mask, Real* __restrict__ grad) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int N = m.N, F = m.F, B = m.B;
  Real g[NQ][3];
  Real qc[NQ], qmax[NQ], qmin[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    g[k][0] = g[k][1] = g[k][2] = 0.0;
    qc[k] = (mask >> k) & 1 ? q[k * N + c] : Real(0.0);
    qmax[k] = qmin[k] = qc[k];
  }
  const int e0 = m.cptr[c], e1 = m.cptr[c + 1];
  for (int e = e0; e < e1; ++e) {
    const int code = m.cface[e];
    const bool isOwn = code >= 0;
    const int f = isOwn ? code : ~code;
    const int o = m.own[f], nb = m.nei[f];
    const int other = isOwn ? nb : o;
    const double wf = m.w[f];
    // the owner adds S sf, the neighbour subtracts it: fold the sign into S
    // (exact) so each component is one multiply-add whichever side this is
    const double sg = isOwn ? 1.0 : -1.0;
    const double S0 = sg * m.Sf[f], S1 = sg * m.Sf[F + f], S2 = sg * m.Sf[2 * F + f];
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      if (!((mask >> k) & 1)) continue;
      const Real qo = q[k * N + other];
      const Real qown = isOwn ? qc[k] : qo, qnei = isOwn ? qo : qc[k];
      const Real sf = wf * (qown - qnei) + qnei;
      g[k][0] = g[k][0] + S0 * sf;
      g[k][1] = g[k][1] + S1 * sf;
      g[k][2] = g[k][2] + S2 * sf;
      if (LIMITED) {
        qmax[k] = omax(qmax[k], qo);
        qmin[k] = omin(qmin[k], qo);
      }
    }
  }
  const int b0 = m.bptr[c], b1 = m.bptr[c + 1];
  for (int e = b0; e < b1; ++e) {
    const int b = m.bface[e];
    const double S0 = m.bSf[b], S1 = m.bSf[B + b], S2 = m.bSf[2 * B + b];
    const int pc = m.bpartner ? m.bpartner[b] : -1;
    if (pc >= 0) {
      // cyclic face: linear interpolation with the partner cell, whose value
      // also bounds the limiter (gaussGrad / cellLimitedGrad on a coupled
      // patch; a scalar field's neighbour values are not rotated)
      const double wb = m.bw[b];
      const bool plag = plag_mode(m, b) != 0;
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        if (!((mask >> k) & 1)) continue;
        const Real qn = plag ? plag_q(m, q, k, b, pc) : q[k * N + pc];
        const Real sf = wb * (qc[k] - qn) + qn;
        g[k][0] = g[k][0] + S0 * sf;
        g[k][1] = g[k][1] + S1 * sf;
        g[k][2] = g[k][2] + S2 * sf;
        if (LIMITED) {
          qmax[k] = omax(qmax[k], qn);
          qmin[k] = omin(qmin[k], qn);
        }
      }
      continue;
    }
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      if (!((mask >> k) & 1)) continue;
      const double v = bq[k * B + b];
      g[k][0] = g[k][0] + S0 * v;
      g[k][1] = g[k][1] + S1 * v;
      g[k][2] = g[k][2] + S2 * v;
      if (LIMITED) {
        qmax[k] = omax(qmax[k], Real(v));
        qmin[k] = omin(qmin[k], Real(v));
      }
    }
  }
  // one FP64 reciprocal per cell instead of a division per component
  const double rV = 1.0 / m.V[c];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    g[k][0] = g[k][0] * rV;
    g[k][1] = g[k][1] * rV;
    g[k][2] = g[k][2] * rV;
  }
  if (LIMITED) {
    // cellLimitedGrad: limiter = min over faces of L(r_f), r_f = maxD/e_f
    // (e_f > SMALL), minD/e_f (e_f < -SMALL) or 1.  min(1, L) is
    // non-decreasing in r >= 0 for both limiters, so the minimum is L of the
    // smallest r, and the smallest r comes from the largest |e_f| of each
    // sign: two divisions per field per cell instead of two per face.
    Real epos[NQ], eneg[NQ];
    unsigned small = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      epos[k] = 0.0;
      eneg[k] = 0.0;
      qmax[k] -= qc[k];
      qmin[k] -= qc[k];
      if (m.limWiden > 0.0) {  // cellLimited coefficient k < 1
        const Real wd = m.limWiden * (qmax[k] - qmin[k]);
        qmax[k] = qmax[k] + wd;
        qmin[k] = qmin[k] - wd;
      }
    }
    // comparisons and extrema through the integer image of the doubles (okey)
    auto faceExtrap = [&](int k, const Real& ex) {
      if (ogt(ex, SMALL))
        epos[k] = omax(epos[k], ex);
      else if (olt(ex, -SMALL))
        eneg[k] = omin(eneg[k], ex);
      else
        small |= 1u << k;
    };
    for (int e = e0; e < e1; ++e) {
      const int code = m.cface[e];
      const bool isOwn = code >= 0;
      const int f = isOwn ? code : ~code;
      const double* d = isOwn ? m.dOwn : m.dNei;
      const double d0 = d[f], d1 = d[F + f], d2 = d[2 * F + f];
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        if (!((mask >> k) & 1)) continue;
        faceExtrap(k, d0 * g[k][0] + d1 * g[k][1] + d2 * g[k][2]);
      }
    }
    for (int e = b0; e < b1; ++e) {
      const int b = m.bface[e];
      const double d0 = m.bdOwn[b], d1 = m.bdOwn[B + b], d2 = m.bdOwn[2 * B + b];
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        if (!((mask >> k) & 1)) continue;
        faceExtrap(k, d0 * g[k][0] + d1 * g[k][1] + d2 * g[k][2]);
      }
    }
    const bool anyFace = (e1 > e0) || (b1 > b0);
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      if (!((mask >> k) & 1) || !anyFace) continue;
      // r = ra / rb (rb > 0): the smaller of maxD/e+ and minD/e- found by
      // cross-multiplication, then one division for the limiter itself
      bool have = false;
      Real ra = 1.0, rb = 1.0;
      if (epos[k] > 0.0) {
        ra = qmax[k];
        rb = epos[k];
        have = true;
      }
      if (eneg[k] < 0.0) {
        const Real a2 = -qmin[k], b2 = -eneg[k];
        if (!have || a2 * rb < ra * b2) {
          ra = a2;
          rb = b2;
        }
        have = true;
      }
      if ((small >> k) & 1) {
        if (!have || ra > rb) {
          ra = 1.0;
          rb = 1.0;
        }
        have = true;
      }
      // Venkatakrishnan (r^2 + 2r)/(r^2 + r + 2) and minmod min(r, 1), capped at 1
      const Real lr = LIMITED == 2 ? (ra * ra + 2 * ra * rb) / (ra * ra + ra * rb + 2 * rb * rb) : ra / rb;
      const Real lim = !have ? Real(1.0) : fmin(1.0, lr);
      g[k][0] = g[k][0] * lim;
      g[k][1] = g[k][1] * lim;
      g[k][2] = g[k][2] * lim;
    }
  }
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    if (!((mask >> k) & 1)) continue;
    grad[(3 * k + 0) * N + c] = g[k][0];
    grad[(3 * k + 1) * N + c] = g[k][1];
    grad[(3 * k + 2) * N + c] = g[k][2];
  }
}

// ------------------------------------------------------------ face fluxes
// MRF = true reads the frame face velocity (moving reference frames); the
// default instance has it as the constant zero, so it costs nothing there
// FP64 residual: three blocks per SM (168 registers) keep more warps in
// flight for the FP64 pipe; the dual-number tangent keeps its registers
template <typename Real = double, bool MRF = false>
__global__ void __launch_bounds__(128, is_fp64<Real> ? 3 : 1) k_face(DevMesh m, ResParams P, const Real* __restrict__ q,
                                              const Real* __restrict__ grad, const double* __restrict__ clin,
                                              const double* __restrict__ nf, Real* __restrict__ fflux,
                                              double* __restrict__ frec, double* __restrict__ flam, int FB) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.F) return;
  const int N = m.N, F = m.F;
  const int o = m.own[f], nb = m.nei[f];
  Real qL[NQ], qR[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    if (P.scheme == ICS_FLUX_ROE && k == Q_C) {
      qL[k] = qR[k] = 0.0;
      continue;
    }
    const Real qo = q[k * N + o], qn = q[k * N + nb];
    const int sch = recon_of(P, k);
    qL[k] = reconstruct(m, sch, k, f, o, nb, qo, qn, grad, +1.0);
    qR[k] = reconstruct(m, sch, k, f, o, nb, qo, qn, grad, -1.0);
  }
  FStateT<Real> L{qL[Q_RHO], qL[Q_P], {qL[Q_UX], qL[Q_UY], qL[Q_UZ]}, qL[Q_E], qL[Q_H], qL[Q_C]};
  FStateT<Real> R{qR[Q_RHO], qR[Q_P], {qR[Q_UX], qR[Q_UY], qR[Q_UZ]}, qR[Q_E], qR[Q_H], qR[Q_C]};
  const double S[3] = {m.Sf[f], m.Sf[F + f], m.Sf[2 * F + f]};
  const double n[3] = {nf[f], nf[F + f], nf[2 * F + f]};
  const double magS = m.magSf[f];
  const double um = MRF ? m.mrfU[f] : 0.0;
  Real out[5];
  if (P.scheme == ICS_FLUX_AUSMPLUSUP)
    flux_ausm(L, R, S, magS, P.lowMach, um, out);
  else if (P.scheme == ICS_FLUX_HLLC)
    flux_hllc(L, R, n, magS, P.gamma, um, out);
  else
    flux_roe(L, R, n, magS, P.gamma, P.entropyFix, um, out);
#pragma unroll
  for (int k = 0; k < 5; ++k) fflux[k * FB + f] = out[k];
  if constexpr (is_fp64<Real>) {  // the tangent needs only the fluxes
    frec[0 * F + f] = qL[Q_UX];
    frec[1 * F + f] = qL[Q_UY];
    frec[2 * F + f] = qL[Q_UZ];
    frec[3 * F + f] = qR[Q_UX];
    frec[4 * F + f] = qR[Q_UY];
    frec[5 * F + f] = qR[Q_UZ];
    frec[6 * F + f] = qL[Q_E];
    frec[7 * F + f] = qR[Q_E];
    // wave speed with linear interpolation (setCoAndDeltaT.H:52-54)
    const double wf = m.w[f];
    const double ci = wf * (clin[o] - clin[nb]) + clin[nb];
    double ui[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double a = q[(Q_UX + k) * N + o], b = q[(Q_UX + k) * N + nb];
      ui[k] = wf * (a - b) + b;
    }
    flam[f] = ci + fabs(dot3(ui, n) - um);
  }
}

__global__ void k_bface(DevMesh m, ResParams P, const double* __restrict__ bq, const double* __restrict__ bclin,
                        const double* __restrict__ bnf, double* __restrict__ fflux, double* __restrict__ flam,
                        double* __restrict__ phiB, int FB) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m.B) return;
  if (m.bpartner && m.bpartner[b] >= 0) return;  // cyclic faces: k_cface
  const int B = m.B, F = m.F;
  double qb[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) qb[k] = bq[k * B + b];
  FState L{qb[Q_RHO], qb[Q_P], {qb[Q_UX], qb[Q_UY], qb[Q_UZ]}, qb[Q_E], qb[Q_H], qb[Q_C]};
  const double S[3] = {m.bSf[b], m.bSf[B + b], m.bSf[2 * B + b]};
  const double n[3] = {bnf[b], bnf[B + b], bnf[2 * B + b]};
  const double magS = m.bmagSf[b];
  const double um = m.mrfU ? m.mrfU[F + b] : 0.0;
  double out[5];
  if (P.scheme == ICS_FLUX_AUSMPLUSUP)
    flux_ausm(L, L, S, magS, P.lowMach, um, out);
  else if (P.scheme == ICS_FLUX_HLLC)
    flux_hllc(L, L, n, magS, P.gamma, um, out);
  else
    flux_roe(L, L, n, magS, P.gamma, P.entropyFix, um, out);
#pragma unroll
  for (int k = 0; k < 5; ++k) fflux[k * FB + F + b] = out[k];
  phiB[b] = out[0];
  flam[F + b] = bclin[b] + fabs(dot3(L.U, n) - um);
}

// Reconstruction on a cyclic face between this side's cell o and the
// partner cell pc: linearUpwind / limitedScheme on a coupled patch.  The
// partner's value enters as it is (the fields reconstructed here are scalar
// fields, U component by component); its gradient vector is rotated into
// this side's frame (patchNeighbourField of the gradient); the partner side
// extrapolates along Cf - C - delta, the TVD ratio uses delta.
template <typename Real>
__device__ __forceinline__ Real reconstruct_cyc(const DevMesh& m, int scheme, int k, int b, int o, int pc,
                                                const Real& qo, const Real& qn, const Real* __restrict__ grad,
                                                const double* R, double dir) {
  const int N = m.N, B = m.B;
  const double wUp = dir > 0 ? 1.0 : 0.0;
  if (scheme == ICS_RECON_UPWIND) return wUp * (qo - qn) + qn;
  Real g0, g1, g2;
  if (dir > 0) {
    g0 = grad[(3 * k) * N + o];
    g1 = grad[(3 * k + 1) * N + o];
    g2 = grad[(3 * k + 2) * N + o];
  } else {
    const Real a0 = grad[(3 * k) * N + pc], a1 = grad[(3 * k + 1) * N + pc], a2 = grad[(3 * k + 2) * N + pc];
    g0 = R[0] * a0 + R[1] * a1 + R[2] * a2;
    g1 = R[3] * a0 + R[4] * a1 + R[5] * a2;
    g2 = R[6] * a0 + R[7] * a1 + R[8] * a2;
  }
  if (scheme == ICS_RECON_VANLEER || scheme == ICS_RECON_MINMOD) {
    const Real gradf = qn - qo;
    const Real gradcf = m.bdelta[b] * g0 + m.bdelta[B + b] * g1 + m.bdelta[2 * B + b] * g2;
    Real r;
    if (fabs(gradcf) >= 1000 * fabs(gradf))
      r = 2 * 1000 * (gradcf >= 0 ? 1.0 : -1.0) * (gradf >= 0 ? 1.0 : -1.0) - 1.0;
    else
      r = 2 * (gradcf / gradf) - 1;
    Real lim;
    if (scheme == ICS_RECON_VANLEER)
      lim = (r + fabs(r)) / (1 + fabs(r));
    else
      lim = fmax(fmin(fmin(r, 1.0), 2.0), 0.0);
    const Real wgt = lim * m.bw[b] + (1.0 - lim) * wUp;
    return wgt * (qo - qn) + qn;
  }
  const double* d = dir > 0 ? m.bdOwn : m.bdNei;
  const Real base = wUp * (qo - qn) + qn;
  return base + (d[b] * g0 + d[B + b] * g1 + d[2 * B + b] * g2);
}

// Flux through the cyclic faces (one thread per face of the list); writes
// the face flux, the boundary mass flux, the wave speed with the coupled
// linear interpolation (velocity rotated: fvc::interpolate of a vector
// field) and the reconstructed states for the Jacobian.
template <typename Real = double, bool MRF = false>
__global__ void __launch_bounds__(128) k_cface(DevMesh m, ResParams P, const Real* __restrict__ q,
                                               const Real* __restrict__ grad, const double* __restrict__ clin,
                                               Real* __restrict__ fflux, double* __restrict__ cfrec,
                                               double* __restrict__ flam, double* __restrict__ phiB, int FB) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.ncyc) return;
  const int N = m.N, F = m.F, B = m.B, nc = m.ncyc;
  const int b = m.cyc_face[i];
  const int o = m.bcell[b], pc = m.bpartner[b];
  const double* R = m.patches[m.bpatch[b]].R;
  Real qL[NQ], qR[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    if (P.scheme == ICS_FLUX_ROE && k == Q_C) {
      qL[k] = qR[k] = 0.0;
      continue;
    }
    const Real qo = q[k * N + o];
    const Real qn = plag_mode(m, b) ? plag_q(m, q, k, b, pc) : q[k * N + pc];
    const int sch = recon_of(P, k);
    qL[k] = reconstruct_cyc(m, sch, k, b, o, pc, qo, qn, grad, R, +1.0);
    qR[k] = reconstruct_cyc(m, sch, k, b, o, pc, qo, qn, grad, R, -1.0);
  }
  FStateT<Real> L{qL[Q_RHO], qL[Q_P], {qL[Q_UX], qL[Q_UY], qL[Q_UZ]}, qL[Q_E], qL[Q_H], qL[Q_C]};
  FStateT<Real> Rs{qR[Q_RHO], qR[Q_P], {qR[Q_UX], qR[Q_UY], qR[Q_UZ]}, qR[Q_E], qR[Q_H], qR[Q_C]};
  const double S[3] = {m.bSf[b], m.bSf[B + b], m.bSf[2 * B + b]};
  const double n[3] = {m.bnf[b], m.bnf[B + b], m.bnf[2 * B + b]};
  const double magS = m.bmagSf[b];
  const double um = MRF ? m.mrfU[F + b] : 0.0;
  Real out[5];
  if (P.scheme == ICS_FLUX_AUSMPLUSUP)
    flux_ausm(L, Rs, S, magS, P.lowMach, um, out);
  else if (P.scheme == ICS_FLUX_HLLC)
    flux_hllc(L, Rs, n, magS, P.gamma, um, out);
  else
    flux_roe(L, Rs, n, magS, P.gamma, P.entropyFix, um, out);
#pragma unroll
  for (int k = 0; k < 5; ++k) fflux[k * FB + F + b] = out[k];
  if constexpr (is_fp64<Real>) {
    phiB[b] = out[0];
    cfrec[0 * nc + i] = qL[Q_UX];
    cfrec[1 * nc + i] = qL[Q_UY];
    cfrec[2 * nc + i] = qL[Q_UZ];
    cfrec[3 * nc + i] = qR[Q_UX];
    cfrec[4 * nc + i] = qR[Q_UY];
    cfrec[5 * nc + i] = qR[Q_UZ];
    cfrec[6 * nc + i] = qL[Q_E];
    cfrec[7 * nc + i] = qR[Q_E];
    const double wb = m.bw[b];
    const bool plag = plag_mode(m, b) != 0;
    const double cn = plag ? plag_q(m, q, Q_C, b, pc) : clin[pc];
    const double ci = wb * (clin[o] - cn) + cn;
    double rpv[3];
    if (plag) {
      plag_vec(m, b, pc, q + Q_UX * N, q + Q_UY * N, q + Q_UZ * N, rpv);
    } else {
      const double Up[3] = {q[Q_UX * N + pc], q[Q_UY * N + pc], q[Q_UZ * N + pc]};
#pragma unroll
      for (int k = 0; k < 3; ++k) rpv[k] = R[3 * k] * Up[0] + R[3 * k + 1] * Up[1] + R[3 * k + 2] * Up[2];
    }
    double ui[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double rp = rpv[k];
      ui[k] = wb * (q[(Q_UX + k) * N + o] - rp) + rp;
    }
    flam[F + b] = ci + fabs(dot3(ui, n) - um);
  }
}

// ------------------------------------------------------------ cell residual
struct CellResParams {
  int ddt;            // ICS_DDT_*
  double rDeltaT, coefft, coefft0, coefft00;
  double serRatio;    // SER factor (setCoAndDeltaT.H:18-26)
  int applySer;
  double coMin, coMax;
};

__device__ __forceinline__ void ddt_matrix(const CellResParams& D, double Vc, double rpdt, double W, double W0,
                                           double W00, double& dg, double& s) {
  if (D.ddt == ICS_DDT_STEADY) {
    dg = 0;
    s = 0;
  } else if (D.ddt == ICS_DDT_EULER) {
    dg = D.rDeltaT * Vc;
    s = D.rDeltaT * W0 * Vc;
  } else {
    dg = (D.coefft * D.rDeltaT) * Vc;
    s = D.rDeltaT * Vc * (D.coefft0 * W0 - D.coefft00 * W00);
  }
  dg += rpdt * Vc;
  s += rpdt * W * Vc;
}

__global__ void __launch_bounds__(128) k_cellres(DevMesh m, CellResParams D, const double* __restrict__ fflux, int FB,
                                                 const double* __restrict__ flam, const double* __restrict__ W,
                                                 const double* __restrict__ W0, const double* __restrict__ W00,
                                                 const double* __restrict__ prim, const double* __restrict__ clin,
                                                 double* __restrict__ pseudoCo, double* __restrict__ rPDT,
                                                 double* __restrict__ ddtCoeff, double* __restrict__ src,
                                                 double* __restrict__ l2cell, const double* __restrict__ fvisc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int N = m.N, F = m.F, B = m.B;
  // viscous terms: laplacian(mu,U), div(tauMC), div(sigmaDotU.S), laplacian(alpha,e),
  // each summed over the faces and divided by V on its own (residualsUpdate.H:24-42)
  double vt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (fvisc) {
    for (int e = m.cptr[c]; e < m.cptr[c + 1]; ++e) {
      const int code = m.cface[e];
      const int f = code >= 0 ? code : ~code;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const double v = fvisc[k * FB + f];
        vt[k] = code >= 0 ? vt[k] + v : vt[k] - v;
      }
    }
    for (int e = m.bptr[c]; e < m.bptr[c + 1]; ++e) {
      const int b = m.bface[e];
#pragma unroll
      for (int k = 0; k < 8; ++k) vt[k] += fvisc[k * FB + F + b];
    }
  }
  double dv[5] = {0, 0, 0, 0, 0};
  double rmax = 0.0;
  const int e0 = m.cptr[c], e1 = m.cptr[c + 1];
  for (int e = e0; e < e1; ++e) {
    const int code = m.cface[e];
    const int f = code >= 0 ? code : ~code;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const double v = fflux[k * FB + f];
      dv[k] = code >= 0 ? dv[k] + v : dv[k] - v;
    }
    rmax = fmax(rmax, m.nodc[f] * flam[f]);
  }
  const int b0 = m.bptr[c], b1 = m.bptr[c + 1];
  for (int e = b0; e < b1; ++e) {
    const int b = m.bface[e];
#pragma unroll
    for (int k = 0; k < 5; ++k) dv[k] += fflux[k * FB + F + b];
    if (m.bpartner && m.bpartner[b] >= 0) {
      // coupled face: nonOrthDeltaCoeffs lambda as for an internal face (setCoAndDeltaT.H:73-87)
      rmax = fmax(rmax, m.bnodc[b] * flam[F + b]);
    } else if (m.patches[m.bpatch[b]].is_wall) {
      const double U0 = prim[2 * N + c], U1 = prim[3 * N + c], U2 = prim[4 * N + c];
      const double bm = m.bmagSf[b];
      const double un = U0 * (m.bSf[b] / bm) + U1 * (m.bSf[B + b] / bm) + U2 * (m.bSf[2 * B + b] / bm);
      const double umb = m.mrfU ? m.mrfU[F + b] : 0.0;
      const double pl = 0.5 * m.bdc[b] * (clin[c] + fabs(un - umb));
      rmax = fmax(rmax, pl);
    }
  }
  const double Vc = m.V[c];
  double r[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) r[k] = -(dv[k] / Vc);
  const double dV0 = (dv[0] / Vc) * Vc;
  l2cell[c] = dV0 * dV0;
  if (fvisc) {
#pragma unroll
    for (int k = 0; k < 3; ++k) r[1 + k] = r[1 + k] + vt[k] / Vc;
#pragma unroll
    for (int k = 0; k < 3; ++k) r[1 + k] = r[1 + k] + vt[3 + k] / Vc;
    r[4] += vt[6] / Vc;
    r[4] += vt[7] / Vc;
  }
  const double rpOld = rPDT[c];
  if (D.ddt != ICS_DDT_STEADY) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      double dg, s;
      const double w = W[5 * c + k];
      ddt_matrix(D, Vc, rpOld, w, W0[5 * c + k], W00[5 * c + k], dg, s);
      r[k] -= (dg * w - s) / Vc;
    }
  }
  if (m.nInst > 1) {
    // Harmonic Balance source -V sum_K D_JK W_K of this cell's instance J
    // (HBZoneTemplates.C:39-92, HBZone.C:520-652 in its zone and with
    // cylCoords), added to R*V (HB residualsUpdate.H:72-74)
    double hb[5] = {0, 0, 0, 0, 0};
    hb_apply(m, c, -Vc, W, hb);
#pragma unroll
    for (int k = 0; k < 5; ++k) src[5 * c + k] = r[k] * Vc + hb[k];
  } else {
#pragma unroll
    for (int k = 0; k < 5; ++k) src[5 * c + k] = r[k] * Vc;
  }
  if (m.mrfOm) {
    // MRF source -(omega x rho U) V on the momentum equations
    // (convectiveFluxScheme.C:123-129), rho U = rho_ * U_
    const double om[3] = {m.mrfOm[c], m.mrfOm[N + c], m.mrfOm[2 * N + c]};
    const double rho = W[5 * c];
    const double rU[3] = {rho * prim[2 * N + c], rho * prim[3 * N + c], rho * prim[4 * N + c]};
    double cr[3];
    cross3(om, rU, cr);
#pragma unroll
    for (int k = 0; k < 3; ++k) src[5 * c + 1 + k] -= cr[k] * Vc;
  }
  double co = pseudoCo[c];
  // stacked independent cases: each case's own SER factor (< 0: none)
  const double ser = m.caseSer ? m.caseSer[m.caseOf[c]] : D.serRatio;
  if (m.caseSer ? ser >= 0.0 : D.applySer) {
    co *= ser;
    co = fmax(fmin(co, D.coMax), D.coMin);
    pseudoCo[c] = co;
  }
  const double rp = rmax / co;
  rPDT[c] = rp;
  double dg, s;
  ddt_matrix(D, Vc, rp, 0.0, 0.0, 0.0, dg, s);
  ddtCoeff[c] = dg / Vc;
}

// ------------------------------------------------------------------ launch
ResParams res_params(const Handle& h) {
  ResParams P;
  P.R = h.cfg.c.R;
  P.Cv = h.cfg.Cv;
  P.gamma = h.cfg.gamma;
  P.cstarFac = 2.0 * (P.gamma - 1.0) / (P.gamma + 1.0);
  P.scheme = h.cfg.c.flux_scheme;
  P.reconRho = h.cfg.c.recon_rho;
  P.reconU = h.cfg.c.recon_U;
  P.reconT = h.cfg.c.recon_T;
  P.lowMach = h.cfg.c.low_mach_ausm;
  P.entropyFix = h.cfg.c.entropy_fix_coeff;
  return P;
}

void launch_fields(Handle& h) {
  const int n = h.m.N > h.m.B ? h.m.N : h.m.B;
  ICS_LAUNCH(h, ICS_K_FIELDS, k_fields<<<grid_for(n, 256), 256, 0, h.stream>>>(h.m.N, h.m.B, h.W, h.prim, h.pB, h.TB, h.UB, res_params(h), h.q,
                                                   h.bq, h.clin, h.clin + h.m.N));
  ICS_CUDA(cudaGetLastError());
}

unsigned grad_mask(const Handle& h, int* limited) {
  unsigned mask = 0;
  int lim = 0;
  const int rs[3] = {h.cfg.c.recon_rho, h.cfg.c.recon_U, h.cfg.c.recon_T};
  const unsigned groups[3] = {(1u << Q_RHO) | (1u << Q_P), (1u << Q_UX) | (1u << Q_UY) | (1u << Q_UZ),
                              (1u << Q_E) | (1u << Q_H) | (1u << Q_C)};
  for (int g = 0; g < 3; ++g) {
    if (rs[g] == ICS_RECON_UPWIND) continue;
    mask |= groups[g];
    if (rs[g] == ICS_RECON_MUSCL_VENKATAKRISHNAN) lim = 2;
    if (rs[g] == ICS_RECON_MUSCL_MINMOD) lim = lim ? lim : 1;
  }
  if (h.cfg.c.flux_scheme == ICS_FLUX_ROE) mask &= ~(1u << Q_C);
  *limited = lim;
  return mask;
}

template <typename Real>
static void launch_grad_t(Handle& h, const Real* q, Real* grad, int kind) {
  int limited = 0;
  const unsigned mask = grad_mask(h, &limited);
  if (!mask) return;
  // groups mixing limited and unlimited schemes are not supported: all
  // reconstructed groups use the same gradient kind
  const int rs[3] = {h.cfg.c.recon_rho, h.cfg.c.recon_U, h.cfg.c.recon_T};
  for (int g = 0; g < 3; ++g) {
    const bool isMuscl = rs[g] == ICS_RECON_MUSCL_VENKATAKRISHNAN || rs[g] == ICS_RECON_MUSCL_MINMOD;
    if (rs[g] != ICS_RECON_UPWIND && (isMuscl != (limited != 0)))
      throw std::string("reconstruction groups must all be TVD or all MUSCL");
    if (isMuscl && rs[g] != (limited == 2 ? ICS_RECON_MUSCL_VENKATAKRISHNAN : ICS_RECON_MUSCL_MINMOD))
      throw std::string("MUSCL groups must share one gradient limiter");
  }
  const int bs = h.tuneGradBs;
  if (limited == 2)
    ICS_LAUNCH(h, kind, k_grad<2, Real><<<grid_for(h.m.N, bs), bs, 0, h.stream>>>(h.m, q, h.bq, mask, grad));
  else if (limited == 1)
    ICS_LAUNCH(h, kind, k_grad<1, Real><<<grid_for(h.m.N, bs), bs, 0, h.stream>>>(h.m, q, h.bq, mask, grad));
  else
    ICS_LAUNCH(h, kind, k_grad<0, Real><<<grid_for(h.m.N, bs), bs, 0, h.stream>>>(h.m, q, h.bq, mask, grad));
  ICS_CUDA(cudaGetLastError());
}

void launch_grad(Handle& h) { launch_grad_t<double>(h, h.q, h.grad, ICS_K_GRAD); }

// The residual-side launch choices of the autotuner: threads per block of
// the face-flux and gradient kernels (64 or 128; both kernels are FP64-pipe
// bound and their occupancy is set by registers), timed with CUDA events on
// the handle's stream at its current state.
void autotune_residual(Handle& h, std::vector<std::pair<std::string, double>>& log) {
  cudaEvent_t e0, e1;
  ICS_CUDA(cudaEventCreate(&e0));
  ICS_CUDA(cudaEventCreate(&e1));
  auto timed = [&](auto&& fn) {
    fn();
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
      ICS_CUDA(cudaEventRecord(e0, h.stream));
      fn();
      ICS_CUDA(cudaEventRecord(e1, h.stream));
      ICS_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      ICS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best = ms < best ? ms : best;
    }
    return (double)best;
  };
  launch_fields(h);
  int bestG = h.tuneGradBs, bestF = h.tuneFaceBs;
  double tg = 1e300, tf = 1e300;
  for (int bs : {64, 128}) {
    h.tuneGradBs = bs;
    const double ms = timed([&]() { launch_grad(h); });
    log.emplace_back("grad_block_" + std::to_string(bs), ms);
    if (ms < tg) tg = ms, bestG = bs;
  }
  h.tuneGradBs = bestG;
  launch_grad(h);
  for (int bs : {64, 128}) {
    h.tuneFaceBs = bs;
    const double ms = timed([&]() { launch_face_flux(h); });
    log.emplace_back("face_block_" + std::to_string(bs), ms);
    if (ms < tf) tf = ms, bestF = bs;
  }
  h.tuneFaceBs = bestF;
  ICS_CUDA(cudaEventDestroy(e0));
  ICS_CUDA(cudaEventDestroy(e1));
}

void launch_face_flux(Handle& h) {
  const int FB = h.m.F + h.m.B;
  const ResParams P = res_params(h);
  if (h.m.F > 0) {
    if (h.m.mrfU)
      ICS_LAUNCH(h, ICS_K_FACE, (k_face<double, true><<<grid_for(h.m.F, h.tuneFaceBs), h.tuneFaceBs, 0, h.stream>>>(
                                    h.m, P, h.q, h.grad, h.clin, h.m.nf, h.fflux, h.frec, h.flam, FB)));
    else
      ICS_LAUNCH(h, ICS_K_FACE, k_face<<<grid_for(h.m.F, h.tuneFaceBs), h.tuneFaceBs, 0, h.stream>>>(h.m, P, h.q, h.grad, h.clin, h.m.nf, h.fflux,
                                                          h.frec, h.flam, FB));
  }
  if (h.m.B > 0)
    ICS_LAUNCH(h, ICS_K_BFACE, k_bface<<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, P, h.bq, h.clin + h.m.N, h.m.bnf, h.fflux,
                                                         h.flam, h.phiB, FB));
  if (h.m.ncyc > 0) {
    if (h.m.mrfU)
      ICS_LAUNCH(h, ICS_K_BFACE, (k_cface<double, true><<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(
                                     h.m, P, h.q, h.grad, h.clin, h.fflux, h.cfrec, h.flam, h.phiB, FB)));
    else
      ICS_LAUNCH(h, ICS_K_BFACE, (k_cface<double, false><<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(
                                     h.m, P, h.q, h.grad, h.clin, h.fflux, h.cfrec, h.flam, h.phiB, FB)));
  }
  ICS_CUDA(cudaGetLastError());
}

void launch_residual(Handle& h, double serRatio, bool applySer) {
  CellResParams D;
  D.ddt = h.cfg.c.ddt_scheme;
  D.rDeltaT = D.coefft = D.coefft0 = D.coefft00 = 0;
  if (D.ddt != ICS_DDT_STEADY) {
    D.rDeltaT = 1.0 / h.cfg.c.delta_t;
    if (D.ddt == ICS_DDT_BACKWARD) {
      const double dt = h.cfg.c.delta_t;
      const double dt0 = h.timeIndex <= 1 ? GREAT : dt;
      D.coefft = 1 + dt / (dt + dt0);
      D.coefft00 = dt * dt / (dt0 * (dt + dt0));
      D.coefft0 = D.coefft + D.coefft00;
    }
  }
  D.serRatio = serRatio;
  D.applySer = applySer ? 1 : 0;
  D.coMin = h.cfg.c.pseudo_co_num_min;
  D.coMax = h.cfg.c.pseudo_co_num_max;
  const int FB = h.m.F + h.m.B;
  ICS_LAUNCH(h, ICS_K_CELLRES, k_cellres<<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m, D, h.fflux, FB, h.flam, h.W, h.W0, h.W00, h.prim,
                                                         h.clin, h.pseudoCo, h.rPDT, h.ddtCoeff, h.src, h.scratch,
                                                         h.cfg.c.viscous ? h.fvisc : nullptr));
  ICS_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------ tangent
// Jacobian-vector product of the residual source src = R V with respect to
// the conservative state, by forward-mode dual numbers through the same
// kernels (derive primitives -> fields -> limited gradients -> face fluxes,
// viscous terms), then the tangent of the cell assembly of k_cellres.  The
// boundary values are held fixed: the boundary-face inviscid fluxes have no
// tangent, the viscous boundary-face terms do (through the interior cell).

__global__ void k_seed(long n, const double* __restrict__ W, const double* __restrict__ v, Dual* __restrict__ tW) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) tW[i] = Dual(W[i], v[i]);
}

// d(src)_c = -sum_f +-d(flux_f) + d(viscous face terms) - dgPhys V_c v_c
//            - V_c sum_K D_JK v_(K,c)   (the pseudo-time terms cancel in R)
__global__ void __launch_bounds__(128) k_src_tangent(DevMesh m, double dgPhys, const Dual* __restrict__ fflux,
                                                     const Dual* __restrict__ fvisc, int FB,
                                                     const double* __restrict__ v, double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  double dv[5] = {0, 0, 0, 0, 0};
  for (int e = m.cptr[c]; e < m.cptr[c + 1]; ++e) {
    const int code = m.cface[e];
    const int f = code >= 0 ? code : ~code;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const double t = fflux[k * FB + f].d;
      dv[k] = code >= 0 ? dv[k] + t : dv[k] - t;
    }
  }
  if (m.bpartner)
    for (int e = m.bptr[c]; e < m.bptr[c + 1]; ++e) {
      const int b = m.bface[e];
      if (m.bpartner[b] < 0) continue;
#pragma unroll
      for (int k = 0; k < 5; ++k) dv[k] += fflux[k * FB + m.F + b].d;
    }
  double r[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) r[k] = -dv[k];
  if (fvisc) {
    double vt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int e = m.cptr[c]; e < m.cptr[c + 1]; ++e) {
      const int code = m.cface[e];
      const int f = code >= 0 ? code : ~code;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const double t = fvisc[k * FB + f].d;
        vt[k] = code >= 0 ? vt[k] + t : vt[k] - t;
      }
    }
    for (int e = m.bptr[c]; e < m.bptr[c + 1]; ++e) {
      const int b = m.bface[e];
#pragma unroll
      for (int k = 0; k < 8; ++k) vt[k] += fvisc[k * FB + m.F + b].d;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) r[1 + k] += vt[k] + vt[3 + k];
    r[4] += vt[6] + vt[7];
  }
  const double Vc = m.V[c];
#pragma unroll
  for (int k = 0; k < 5; ++k) r[k] -= dgPhys * Vc * v[5 * c + k];
  if (m.mrfOm) {  // the MRF source is linear in rho U
    const int N = m.N;
    const double om[3] = {m.mrfOm[c], m.mrfOm[N + c], m.mrfOm[2 * N + c]};
    const double vU[3] = {v[5 * c + 1], v[5 * c + 2], v[5 * c + 3]};
    double cr[3];
    cross3(om, vU, cr);
#pragma unroll
    for (int k = 0; k < 3; ++k) r[1 + k] -= cr[k] * Vc;
  }
  if (m.nInst > 1) hb_apply(m, c, -Vc, v, r);  // the HB source is linear in W
#pragma unroll
  for (int k = 0; k < 5; ++k) out[5 * c + k] = r[k];
}

void launch_derive_tangent(Handle& h, const Dual* W, Dual* prim);
void launch_viscous_tangent(Handle& h, const Dual* W, const Dual* prim, Dual* vc, Dual* fv);

void launch_residual_tangent(Handle& h, const double* v, double* out) {
  const int N = h.m.N, FB = h.m.F + h.m.B;
  Dual* tW = (Dual*)h.tW;
  Dual* tprim = (Dual*)h.tprim;
  Dual* tq = (Dual*)h.tq;
  Dual* tgrad = (Dual*)h.tgrad;
  Dual* tflux = (Dual*)h.tflux;
  const ResParams P = res_params(h);
  // the boundary field values (bq) of the current boundary state
  launch_fields(h);
  ICS_LAUNCH(h, ICS_K_TANGENT, k_seed<<<grid_for(5L * N, 256), 256, 0, h.stream>>>(5L * N, h.W, v, tW));
  launch_derive_tangent(h, tW, tprim);
  ICS_LAUNCH(h, ICS_K_TANGENT, k_fields<Dual><<<grid_for(N, 256), 256, 0, h.stream>>>(N, 0, tW, tprim, nullptr, nullptr,
                                                                                      nullptr, P, tq, nullptr, nullptr,
                                                                                      nullptr));
  launch_grad_t<Dual>(h, tq, tgrad, ICS_K_TANGENT);
  if (h.m.F > 0) {
    if (h.m.mrfU)
      ICS_LAUNCH(h, ICS_K_TANGENT, (k_face<Dual, true><<<grid_for(h.m.F, 128), 128, 0, h.stream>>>(
                                       h.m, P, tq, tgrad, nullptr, h.m.nf, tflux, nullptr, nullptr, FB)));
    else
      ICS_LAUNCH(h, ICS_K_TANGENT, k_face<Dual><<<grid_for(h.m.F, 128), 128, 0, h.stream>>>(h.m, P, tq, tgrad, nullptr,
                                                                                            h.m.nf, tflux, nullptr,
                                                                                            nullptr, FB));
  }
  if (h.m.ncyc > 0) {  // the cyclic faces depend on the cells of both sides
    if (h.m.mrfU)
      ICS_LAUNCH(h, ICS_K_TANGENT, (k_cface<Dual, true><<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(
                                       h.m, P, tq, tgrad, nullptr, tflux, nullptr, nullptr, nullptr, FB)));
    else
      ICS_LAUNCH(h, ICS_K_TANGENT, (k_cface<Dual, false><<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(
                                       h.m, P, tq, tgrad, nullptr, tflux, nullptr, nullptr, nullptr, FB)));
  }
  Dual* tfv = nullptr;
  if (h.cfg.c.viscous) {
    tfv = (Dual*)h.tfv;
    launch_viscous_tangent(h, tW, tprim, (Dual*)h.tvc, tfv);
  }
  double dgPhys = 0.0;
  if (h.cfg.c.ddt_scheme == ICS_DDT_EULER) dgPhys = 1.0 / h.cfg.c.delta_t;
  if (h.cfg.c.ddt_scheme == ICS_DDT_BACKWARD) {
    const double dt = h.cfg.c.delta_t;
    const double dt0 = h.timeIndex <= 1 ? GREAT : dt;
    dgPhys = (1 + dt / (dt + dt0)) / dt;
  }
  ICS_LAUNCH(h, ICS_K_TANGENT, k_src_tangent<<<grid_for(N, 128), 128, 0, h.stream>>>(h.m, dgPhys, tflux, tfv, FB, v,
                                                                                     out));
  ICS_CUDA(cudaGetLastError());
}

// ------------------------------------------------------- passive scalar
// calculateScalarTransport.H: rho s advected with a Roe-averaged upwind flux
// (Harten's fix), laplacian(D, s) for viscous cases, and the 1x1-block
// matrix: convective blocks from the reconstructed normal velocities, LF
// dissipation |interpolate(U).n|, geometric-boundary diagonal, viscous
// stabilisation 0.5 D/rho_f |S| deltaCoeffs, dual-time diagonal.
// sface layout [5][F+B]: 0 flux - laplacian, 1 upper, 2 lower, 3 owner diag,
// 4 neighbour diag (boundary faces: 0 and 3 only).
__global__ void __launch_bounds__(128) k_scalar_face(DevMesh m, ResParams P, int reconS, double Ds, int viscous,
                                                     const double* __restrict__ q, const double* __restrict__ grad,
                                                     const double* __restrict__ s, const double* __restrict__ sgrad,
                                                     const double* __restrict__ sgradL, double* __restrict__ out,
                                                     int FB) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.F) return;
  const int N = m.N, F = m.F;
  const int o = m.own[f], nb = m.nei[f];
  const double sl = reconstruct(m, reconS, 0, f, o, nb, s[o], s[nb], sgrad, +1.0);
  const double sr = reconstruct(m, reconS, 0, f, o, nb, s[o], s[nb], sgrad, -1.0);
  const double rl = reconstruct(m, P.reconRho, Q_RHO, f, o, nb, q[Q_RHO * N + o], q[Q_RHO * N + nb], grad, +1.0);
  const double rr = reconstruct(m, P.reconRho, Q_RHO, f, o, nb, q[Q_RHO * N + o], q[Q_RHO * N + nb], grad, -1.0);
  double Ul[3], Ur[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int qk = Q_UX + k;
    Ul[k] = reconstruct(m, P.reconU, qk, f, o, nb, q[qk * N + o], q[qk * N + nb], grad, +1.0);
    Ur[k] = reconstruct(m, P.reconU, qk, f, o, nb, q[qk * N + o], q[qk * N + nb], grad, -1.0);
  }
  const double ms = m.magSf[f];
  const double n[3] = {m.nf[f], m.nf[F + f], m.nf[2 * F + f]};
  const double rSl = rl * sl, rSr = rr * sr;
  const double coefR = sqrt(fmax(VSMALL, rr) / fmax(VSMALL, rl));
  double roeU[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) roeU[k] = (coefR * Ur[k] + Ul[k]) / (coefR + 1.0);
  const double um = m.mrfU ? m.mrfU[f] : 0.0;
  const double uProj = dot3(roeU, n) - um;
  double lam = fabs(uProj);
  const double eps = 0.05 * lam;
  if (lam < eps) lam = (lam * lam + eps * eps) / (2.0 * eps);
  const double unl = dot3(Ul, n), unr = dot3(Ur, n);
  double ph = -0.5 * ms * lam * (rSr - rSl);
  ph += 0.5 * ms * (rl * unl * sl + rr * unr * sr);
  ph -= 0.5 * ms * um * (rSl + rSr);
  const double wf = m.w[f];
  // LF dissipation with the linearly interpolated cell velocity
  double Uf[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double a = q[(Q_UX + k) * N + o], b = q[(Q_UX + k) * N + nb];
    Uf[k] = wf * (a - b) + b;
  }
  const double d = 0.5 * ms * fabs(dot3(Uf, n) - um);
  double stab = 0.0, lap = 0.0;
  if (viscous) {
    const double nodc = m.nodc[f];
    double kc[3], gf[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      kc[k] = n[k] - m.dCC[k * F + f] * nodc;
      gf[k] = wf * (sgradL[k * N + o] - sgradL[k * N + nb]) + sgradL[k * N + nb];
    }
    lap = (Ds * ms) * (nodc * (s[nb] - s[o]) + dot3(kc, gf));
    const double rhof = wf * (q[Q_RHO * N + o] - q[Q_RHO * N + nb]) + q[Q_RHO * N + nb];
    stab = 0.5 * (Ds / rhof) * ms * m.dc[f];
  }
  double up = 0.5 * ms * unr, lo = -0.5 * ms * unl;
  if (um != 0.0) {  // -div(w, u_MRF |S|) (calculateScalarTransport.H:217-219)
    const double phm = um * ms;
    up -= phm * (1.0 - wf);
    lo -= -phm * wf;
  }
  out[f] = ph - lap;
  out[FB + f] = up - d - stab;
  out[2 * FB + f] = lo - d - stab;
  out[3 * FB + f] = -lo + d + stab;
  out[4 * FB + f] = -up + d + stab;
}

__global__ void k_scalar_bface(DevMesh m, double Ds, int viscous, const double* __restrict__ bq,
                               const double* __restrict__ q, const double* __restrict__ s,
                               const double* __restrict__ sB, const int* __restrict__ sFixed,
                               double* __restrict__ out, int FB) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m.B) return;
  if (m.bpartner && m.bpartner[b] >= 0) return;  // cyclic faces: k_scalar_cface
  const int B = m.B, F = m.F, N = m.N;
  const int ci = m.bcell[b];
  const double ms = m.bmagSf[b];
  const double S[3] = {m.bSf[b], m.bSf[B + b], m.bSf[2 * B + b]};
  const double n[3] = {m.bnf[b], m.bnf[B + b], m.bnf[2 * B + b]};
  const double rb = bq[Q_RHO * B + b];
  const double Ub[3] = {bq[Q_UX * B + b], bq[Q_UY * B + b], bq[Q_UZ * B + b]};
  const double sb = sB[b];
  const double rS = rb * sb;
  const double coefR = sqrt(fmax(VSMALL, rb) / fmax(VSMALL, rb));
  double roeU[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) roeU[k] = (coefR * Ub[k] + Ub[k]) / (coefR + 1.0);
  const double um = m.mrfU ? m.mrfU[F + b] : 0.0;
  double lam = fabs(dot3(roeU, n) - um);
  const double eps = 0.05 * lam;
  if (lam < eps) lam = (lam * lam + eps * eps) / (2.0 * eps);
  const double un = dot3(Ub, n);
  double ph = -0.5 * ms * lam * (rS - rS);
  ph += 0.5 * ms * (rb * un * sb + rb * un * sb);
  ph -= 0.5 * ms * um * (rS + rS);
  double lap = 0.0;
  if (viscous) lap = (Ds * ms) * ((sb - s[ci]) * m.bdc[b]);
  out[F + b] = ph - lap;
  // dissipation |U_b.n| and rho_B (U_B . S_B) valueInternalCoeffs / rho_I
  const double vic = sFixed[m.bpatch[b]] ? 0.0 : 1.0;
  const double flux = rb * (dot3(Ub, S) - um * ms) * vic;
  out[3 * FB + F + b] = 0.5 * ms * fabs(un - um) + flux * (1.0 / q[Q_RHO * N + ci]);
}

// Cyclic faces of the passive scalar: the face between this side's cell and
// the partner (s, rho and the U components reconstructed as in k_cface), the
// coupled half of insertBlock / the MRF divergence / the dissipation block,
// the interface coefficient (no rotation: a scalar unknown) in the upper slot.
__global__ void __launch_bounds__(128) k_scalar_cface(DevMesh m, ResParams P, int reconS,
                                                      const double* __restrict__ q, const double* __restrict__ grad,
                                                      const double* __restrict__ bq, const double* __restrict__ s,
                                                      const double* __restrict__ sgrad, double* __restrict__ out,
                                                      int FB) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.ncyc) return;
  const int N = m.N, F = m.F, B = m.B;
  const int b = m.cyc_face[i];
  const int o = m.bcell[b], pc = m.bpartner[b];
  const double* R = m.patches[m.bpatch[b]].R;
  const double sl = reconstruct_cyc(m, reconS, 0, b, o, pc, s[o], s[pc], sgrad, R, +1.0);
  const double sr = reconstruct_cyc(m, reconS, 0, b, o, pc, s[o], s[pc], sgrad, R, -1.0);
  const bool plag = plag_mode(m, b) != 0;
  const double qo = q[Q_RHO * N + o], qn = plag ? plag_q(m, q, Q_RHO, b, pc) : q[Q_RHO * N + pc];
  const double rl = reconstruct_cyc(m, P.reconRho, Q_RHO, b, o, pc, qo, qn, grad, R, +1.0);
  const double rr = reconstruct_cyc(m, P.reconRho, Q_RHO, b, o, pc, qo, qn, grad, R, -1.0);
  double Ul[3], Ur[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int qk = Q_UX + k;
    const double un = plag ? plag_q(m, q, qk, b, pc) : q[qk * N + pc];
    Ul[k] = reconstruct_cyc(m, P.reconU, qk, b, o, pc, q[qk * N + o], un, grad, R, +1.0);
    Ur[k] = reconstruct_cyc(m, P.reconU, qk, b, o, pc, q[qk * N + o], un, grad, R, -1.0);
  }
  const double ms = m.bmagSf[b];
  const double n[3] = {m.bnf[b], m.bnf[B + b], m.bnf[2 * B + b]};
  const double rSl = rl * sl, rSr = rr * sr;
  const double coefR = sqrt(fmax(VSMALL, rr) / fmax(VSMALL, rl));
  double roeU[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) roeU[k] = (coefR * Ur[k] + Ul[k]) / (coefR + 1.0);
  const double um = m.mrfU ? m.mrfU[F + b] : 0.0;
  double lam = fabs(dot3(roeU, n) - um);
  const double eps = 0.05 * lam;
  if (lam < eps) lam = (lam * lam + eps * eps) / (2.0 * eps);
  const double unl = dot3(Ul, n), unr = dot3(Ur, n);
  double ph = -0.5 * ms * lam * (rSr - rSl);
  ph += 0.5 * ms * (rl * unl * sl + rr * unr * sr);
  ph -= 0.5 * ms * um * (rSl + rSr);
  // LF dissipation with the coupled patch value of U (the rotated interpolate)
  const double Ub[3] = {bq[Q_UX * B + b], bq[Q_UY * B + b], bq[Q_UZ * B + b]};
  const double d = 0.5 * ms * fabs(dot3(Ub, n) - um);
  double up = 0.5 * ms * unr, lo = -0.5 * ms * unl;
  if (um != 0.0) {
    const double phm = um * ms, wb = m.bw[b];
    up -= phm * (1.0 - wb);
    lo -= -phm * wb;
  }
  out[F + b] = ph;
  out[FB + F + b] = up - d;
  out[3 * FB + F + b] = -lo + d;
}

__global__ void __launch_bounds__(128) k_scalar_rows(DevMesh m, CellResParams D, const double* __restrict__ face,
                                                     int FB, const double* __restrict__ rhoS,
                                                     const double* __restrict__ rhoS0,
                                                     const double* __restrict__ rhoS00, const double* __restrict__ rPDT,
                                                     double* __restrict__ src, double* __restrict__ blk,
                                                     double* __restrict__ dg, double* __restrict__ rD,
                                                     int* __restrict__ status) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int F = m.F;
  double dv = 0.0, diag = 0.0;
  for (int e = m.cptr[c]; e < m.cptr[c + 1]; ++e) {
    const int code = m.cface[e];
    const int f = code >= 0 ? code : ~code;
    dv = code >= 0 ? dv + face[f] : dv - face[f];
    diag += code >= 0 ? face[3 * FB + f] : face[4 * FB + f];
  }
  for (int e = m.bptr[c]; e < m.bptr[c + 1]; ++e) {
    const int b = m.bface[e];
    dv += face[F + b];
    diag += face[3 * FB + F + b];
  }
  const double Vc = m.V[c];
  double r = -(dv / Vc);
  double dgt, st;
  ddt_matrix(D, Vc, rPDT[c], rhoS[c], rhoS0[c], rhoS00[c], dgt, st);
  if (D.ddt != ICS_DDT_STEADY) r -= (dgt * rhoS[c] - st) / Vc;
  src[c] = r * Vc;
  diag += dgt;
  // slots in face order: an owner-side face gives the upper coefficient
  const int s = c >> 5, lane = c & 31;
  const int base = m.slot_base[s];
  for (int t = 0; t < m.nslot[c]; ++t) {
    const int code = m.sface[(base + t) * 32 + lane];
    const int f = code >= 0 ? code : ~code;
    blk[(size_t)(base + t) * 32 + lane] = code >= 0 ? face[FB + f] : face[2 * FB + f];
  }
  dg[c] = diag;
  const double r1 = 1.0 / fmax(1.0 / GREAT, fabs(diag));
  if (!(r1 >= VSMALL)) atomicOr(status, 1);
  rD[c] = r1;
}

__global__ void k_scalar_update(DevMesh m, const double* __restrict__ dx, const double* __restrict__ rho,
                                double* __restrict__ rhoS, double* __restrict__ s) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  rhoS[c] += dx[c];
  s[c] = rhoS[c] / rho[c];
}

__global__ void k_scalar_bc(DevMesh m, const double* __restrict__ s, const int* __restrict__ sFixed,
                            const double* __restrict__ sValue, double* __restrict__ sB) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m.B) return;
  const int pi = m.bpatch[b];
  sB[b] = sFixed[pi] ? sValue[pi] : s[m.bcell[b]];
  if (m.bpartner && m.bpartner[b] >= 0) {  // coupled evaluate
    const int pc = m.bpartner[b];
    sB[b] = m.bw[b] * (s[m.bcell[b]] - s[pc]) + s[pc];
  }
}

static CellResParams ddt_params(const Handle& h) {
  CellResParams D;
  D.ddt = h.cfg.c.ddt_scheme;
  D.rDeltaT = D.coefft = D.coefft0 = D.coefft00 = 0;
  D.serRatio = 1;
  D.applySer = 0;
  D.coMin = D.coMax = 0;
  if (D.ddt != ICS_DDT_STEADY) {
    D.rDeltaT = 1.0 / h.cfg.c.delta_t;
    if (D.ddt == ICS_DDT_BACKWARD) {
      const double dt = h.cfg.c.delta_t;
      const double dt0 = h.timeIndex <= 1 ? GREAT : dt;
      D.coefft = 1 + dt / (dt + dt0);
      D.coefft00 = dt * dt / (dt0 * (dt + dt0));
      D.coefft0 = D.coefft + D.coefft00;
    }
  }
  return D;
}

void launch_scalar_assembly(Handle& h) {
  const int N = h.m.N, F = h.m.F, B = h.m.B, FB = F + B;
  const ResParams P = res_params(h);
  // flow fields and reconstruction gradients at the current state
  launch_fields(h);
  launch_grad(h);
  // s gradient for its reconstruction scheme, and a plain Gauss one for the
  // laplacian's non-orthogonal correction
  const int rs = h.reconS;
  const int lim = rs == ICS_RECON_MUSCL_VENKATAKRISHNAN ? 2 : (rs == ICS_RECON_MUSCL_MINMOD ? 1 : 0);
  if (rs != ICS_RECON_UPWIND) {
    if (lim == 2)
      ICS_LAUNCH(h, ICS_K_PASSIVE, k_grad<2, double><<<grid_for(N, 128), 128, 0, h.stream>>>(h.m, h.ss, h.ssB, 1u, h.sgrad));
    else if (lim == 1)
      ICS_LAUNCH(h, ICS_K_PASSIVE, k_grad<1, double><<<grid_for(N, 128), 128, 0, h.stream>>>(h.m, h.ss, h.ssB, 1u, h.sgrad));
    else
      ICS_LAUNCH(h, ICS_K_PASSIVE, k_grad<0, double><<<grid_for(N, 128), 128, 0, h.stream>>>(h.m, h.ss, h.ssB, 1u, h.sgrad));
  }
  const int viscous = h.cfg.c.viscous ? 1 : 0;
  if (viscous)
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_grad<0, double><<<grid_for(N, 128), 128, 0, h.stream>>>(h.m, h.ss, h.ssB, 1u, h.sgradL));
  if (F)
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_scalar_face<<<grid_for(F, 128), 128, 0, h.stream>>>(
                                     h.m, P, rs, h.Ds, viscous, h.q, h.grad, h.ss, h.sgrad, h.sgradL, h.sface, FB));
  if (B)
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_scalar_bface<<<grid_for(B, 128), 128, 0, h.stream>>>(
                                     h.m, h.Ds, viscous, h.bq, h.q, h.ss, h.ssB, h.sFixed, h.sface, FB));
  if (h.m.ncyc)
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_scalar_cface<<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(
                                     h.m, P, rs, h.q, h.grad, h.bq, h.ss, h.sgrad, h.sface, FB));
  ICS_LAUNCH(h, ICS_K_PASSIVE, k_scalar_rows<<<grid_for(N, 128), 128, 0, h.stream>>>(
                                   h.m, ddt_params(h), h.sface, FB, h.srhoS, h.srhoS0, h.srhoS00, h.rPDT, h.ssrc,
                                   h.sblk, h.sdg, h.srD, &h.ks->status));
  ICS_CUDA(cudaGetLastError());
}

void launch_scalar_update(Handle& h, const double* dx) {
  ICS_LAUNCH(h, ICS_K_PASSIVE, k_scalar_update<<<grid_for(h.m.N, 256), 256, 0, h.stream>>>(h.m, dx, h.q, h.srhoS, h.ss));
  if (h.m.B)
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_scalar_bc<<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, h.ss, h.sFixed, h.sValue, h.ssB));
  ICS_CUDA(cudaGetLastError());
}

void launch_scalar_bc(Handle& h) {
  if (h.m.B)
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_scalar_bc<<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, h.ss, h.sFixed, h.sValue, h.ssB));
  ICS_CUDA(cudaGetLastError());
}

}  // namespace ics
