// Jacobian assembly into the sliced-ELL block matrix.
//
// Row-parallel: the thread of cell c writes its whole row (diagonal block and
// one block per internal face), so every store is coalesced across the warp
// and no atomics are needed.  For face f the reference inserts
//     upper_f = 0.5|S| A(W_R) - 0.5|S| lambda I   (row own, column nei)
//     lower_f = -0.5|S| A(W_L) - 0.5|S| lambda I  (row nei, column own)
// and the diagonal is the negative column sum of the off-diagonal blocks
// (LduMatrix::negSumDiag), plus the boundary dissipation, the boundary
// Jacobian and the temporal term.  The off-diagonal slot is stored factored
// (blocks.cuh: the side's state, the signed scaled normal and the identity
// multiple); the diagonal needs the other side's Jacobian, which the cell
// evaluates entry by entry.  In mixed precision this arithmetic runs in FP32.
//
// Reference: convectiveFluxScheme::addFluxTerms (convectiveFluxScheme.C:374-484),
// addDissipationJacobian (:487-534), addBoundaryTerms with boundaryJacobian
// (:47-120, :219-355), addTemporalTerms (:358-369); blockFvMatrix::insertBlock
// and insertDissipationBlock (blockFvMatrix.C:211-326); LU-SGS scalar
// diagonal (lusgs.C:50-127).
#include "blocks.cuh"
#include "flux.cuh"
#include "hb.cuh"
#include "ics_internal.cuh"

namespace ics {

// Euler flux Jacobian entry (row i, column j) of state (U, E) for normal n.
template <typename T>
struct EulerJ {
  T U[3], n[3], theta, a1, a2, projU, g;
  __device__ __forceinline__ void init(T gamma, const T* u, T E, const T* nn) {
    g = gamma;
    for (int k = 0; k < 3; ++k) {
      U[k] = u[k];
      n[k] = nn[k];
    }
    theta = T(0.5) * (g - T(1)) * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
    a1 = g * E - theta;
    a2 = g - T(1);
    projU = U[0] * n[0] + U[1] * n[1] + U[2] * n[2];
  }
  __device__ __forceinline__ T entry(int i, int j) const {
    if (i == 0) return j == 0 ? T(0) : (j == 4 ? T(0) : n[j - 1]);
    if (i == 4) {
      if (j == 0) return projU * (theta - a1);
      if (j == 4) return g * projU;
      return n[j - 1] * a1 - a2 * U[j - 1] * projU;
    }
    const int r = i - 1;
    if (j == 0) return n[r] * theta - U[r] * projU;
    if (j == 4) return n[r] * a2;
    const int cc = j - 1;
    return U[r] * n[cc] - a2 * n[r] * U[cc] + (r == cc ? projU : T(0));
  }
};

// The five laplacian fields of the non-LF viscous Jacobian at one state
// (viscousFluxScheme.C:259-267): -U/rho on momentum by rho and energy by rhoU,
// 1/rho on momentum by rhoU (x I) and energy by rhoE, -E/rho + |U|^2/rho on
// energy by rho, with E = he(T) + 0.5|U|^2.
struct ViscLapField {
  double mUr[3], ir, eR;
  __device__ __forceinline__ void init(double rho, const double* U, double T, double Cv) {
    const double u2 = dot3(U, U);
    const double E = Cv * T + 0.5 * u2;
    for (int k = 0; k < 3; ++k) mUr[k] = -U[k] / rho;
    ir = 1.0 / rho;
    eR = -E / rho + u2 / rho;
  }
  // entry (i, j) of the five laplacians for coefficients mg (mu) and ag (alphaEff)
  __device__ __forceinline__ double entry(int i, int j, double mg, double ag) const {
    if (i >= 1 && i <= 3) {
      if (j == 0) return mUr[i - 1] * mg;
      if (j == i) return ir * mg;
      return 0.0;
    }
    if (i == 4) {
      if (j == 0) return eR * ag;
      if (j == 4) return ir * ag;
      return mUr[j - 1] * ag;
    }
    return 0.0;
  }
};

// Boundary diagonal contribution of one boundary face (addBoundaryTerms and
// the boundary part of insertDissipationBlock), FP64, [25][B].  vj (non-LF
// viscous Jacobian only): the patch mu and alphaEff, [2][F+B].
__global__ void k_jac_boundary(DevMesh m, double R, double Cv, double gamma, const double* __restrict__ W,
                               const double* __restrict__ prim, const double* __restrict__ pB,
                               const double* __restrict__ TB, const double* __restrict__ UBv,
                               const double* __restrict__ phiB, const double* __restrict__ flam,
                               double* __restrict__ bjac, const double* __restrict__ vj) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m.B) return;
  if (m.bpartner && m.bpartner[b] >= 0) return;  // cyclic faces: k_jac_cyclic
  const int B = m.B, N = m.N;
  const Patch pt = m.patches[m.bpatch[b]];
  const int ci = m.bcell[b];
  const double bm = m.bmagSf[b];
  const double SfB[3] = {m.bSf[b], m.bSf[B + b], m.bSf[2 * B + b]};
  const double nf[3] = {SfB[0] / bm, SfB[1] / bm, SfB[2] / bm};
  double pV = 1, tV = 1, uV[3] = {1, 1, 1};
  switch (pt.kind) {
    case ICS_PATCH_SLIP:
      for (int k = 0; k < 3; ++k) uV[k] = 1 - fabs(nf[k]);
      break;
    case ICS_PATCH_FIXED:
      pV = 0;
      tV = 0;
      uV[0] = uV[1] = uV[2] = 0;
      break;
    case ICS_PATCH_PRESSURE_OUTLET: pV = 0; break;
    case ICS_PATCH_TOTAL_INLET:
      pV = 0;
      tV = 0;
      if (phiB[b] < 0)
        for (int k = 0; k < 3; ++k) uV[k] = nf[k] * nf[k];
      break;
    case ICS_PATCH_ISOTHERMAL_WALL:
      tV = 0;
      uV[0] = uV[1] = uV[2] = 0;
      break;
    default: break;
  }
  const double TBb = TB[b], pBb = pB[b];
  const double rhoB = (1.0 / (R * TBb)) * pBb;
  const double UB[3] = {UBv[b], UBv[B + b], UBv[2 * B + b]};
  const double umb = m.mrfU ? m.mrfU[m.F + b] : 0.0;  // MRF frame velocity (convectiveFluxScheme.C:94)
  const double UrelBdotSf = dot3(UB, SfB) - umb * bm;
  const double rhoEB = rhoB * (Cv * TBb + 0.5 * dot3(UB, UB));
  double SuV[3], dCdU[3], dMdp[3], dMdT[3], dEdU[3], dMdUDiag[3];
  double dMdU[3][3];
  const double dCdp = rhoB / pBb * UrelBdotSf * pV;
  const double dCdT = -rhoB / TBb * UrelBdotSf * tV;
  for (int k = 0; k < 3; ++k) {
    SuV[k] = SfB[k] * uV[k];
    dCdU[k] = rhoB * SuV[k];
    dMdp[k] = (rhoB / pBb * UB[k] * UrelBdotSf + SfB[k]) * pV;
    dMdUDiag[k] = rhoB * UrelBdotSf * uV[k];
    dMdT[k] = -rhoB / TBb * UB[k] * UrelBdotSf * tV;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) dMdU[i][j] = (rhoB * UB[i]) * SuV[j];
  for (int i = 0; i < 3; ++i) dMdU[i][i] += dMdUDiag[i];
  const double dEdp = (rhoEB / pBb * UrelBdotSf + dot3(UB, SfB)) * pV;
  for (int k = 0; k < 3; ++k) dEdU[k] = SuV[k] * (rhoEB + pBb) + rhoB * UrelBdotSf * (UB[k] * uV[k]);
  const double dEdT = UrelBdotSf * (rhoB * Cv - rhoEB / TBb) * tV;
  // interior derivatives
  const double rhoI = W[5 * ci], rhoEI = W[5 * ci + 4];
  const double UI[3] = {prim[2 * N + ci], prim[3 * N + ci], prim[4 * N + ci]};
  const double magU2 = dot3(UI, UI);
  const double dPdRho = 0.5 * (gamma - 1) * magU2;
  double dUdRho[3], dPdRhoU[3], dTdRhoU[3];
  for (int k = 0; k < 3; ++k) {
    dUdRho[k] = -1.0 * UI[k] / rhoI;
    dPdRhoU[k] = -(gamma - 1) * UI[k];
    dTdRhoU[k] = -1.0 * UI[k] / (Cv * rhoI);
  }
  const double dTdRho = -1.0 / (Cv * rhoI) * (rhoEI / rhoI - magU2);
  const double dUdRhoU = 1.0 / rhoI;
  const double dPdRhoE = gamma - 1;
  const double dTdRhoE = 1.0 / (Cv * rhoI);
  double D[25];
  for (int k = 0; k < 25; ++k) D[k] = 0.0;
  D[0] = dCdp * dPdRho + dot3(dCdU, dUdRho) + dCdT * dTdRho;
  for (int j = 0; j < 3; ++j) D[1 + j] = dCdp * dPdRhoU[j] + dCdU[j] * dUdRhoU + dCdT * dTdRhoU[j];
  D[4] = dCdp * dPdRhoE + 0.0 + dCdT * dTdRhoE;
  for (int i = 0; i < 3; ++i) {
    D[5 * (1 + i)] = dMdp[i] * dPdRho + (dMdU[i][0] * dUdRho[0] + dMdU[i][1] * dUdRho[1] + dMdU[i][2] * dUdRho[2]) +
                     dMdT[i] * dTdRho;
    for (int j = 0; j < 3; ++j)
      D[5 * (1 + i) + 1 + j] = dMdp[i] * dPdRhoU[j] + dMdU[i][j] * dUdRhoU + dMdT[i] * dTdRhoU[j];
    D[5 * (1 + i) + 4] = dMdp[i] * dPdRhoE + 0.0 + dMdT[i] * dTdRhoE;
  }
  D[20] = dEdp * dPdRho + dot3(dEdU, dUdRho) + dEdT * dTdRho;
  for (int j = 0; j < 3; ++j) D[21 + j] = dEdp * dPdRhoU[j] + dEdU[j] * dUdRhoU + dEdT * dTdRhoU[j];
  D[24] = dEdp * dPdRhoE + 0.0 + dEdT * dTdRhoE;
  // boundary dissipation 0.5 |S_b| lambda_b on the diagonal entries
  const double d = 0.5 * bm * flam[m.F + b];
  for (int q = 0; q < 5; ++q) D[6 * q] += d;
  if (vj) {
    // non-LF viscous boundary terms (viscousFluxScheme.C:41-86, 120-215):
    // dMomFlux/dU = diag(-mu_b uGIC |S|), dEnergyFlux/dT = -alphaEff_b Cv TGIC |S|
    // with gradientInternalCoeffs fixedValue -dc, zeroGradient 0, slip -dc |n_k|,
    // pressureInletOutletVelocity -dc sqrt(|1 - n_k^2|) on inflow faces
    const double dcb = m.bdc[b];
    double uG[3] = {0.0, 0.0, 0.0}, tG = 0.0;
    switch (pt.kind) {
      case ICS_PATCH_SLIP:
        for (int k = 0; k < 3; ++k) uG[k] = -dcb * fabs(nf[k]);
        break;
      case ICS_PATCH_FIXED:
      case ICS_PATCH_ISOTHERMAL_WALL:
        uG[0] = uG[1] = uG[2] = -dcb;
        tG = -dcb;
        break;
      case ICS_PATCH_TOTAL_INLET:
        if (phiB[b] < 0)
          for (int k = 0; k < 3; ++k) uG[k] = -dcb * sqrt(fabs(1.0 - nf[k] * nf[k]));
        tG = -dcb;
        break;
      default: break;
    }
    const int FB = m.F + B;
    const double muB = vj[m.F + b], alB = vj[FB + m.F + b];
    const double EI = Cv * prim[N + ci] + 0.5 * magU2;
    const double dEvdT = -alB * Cv * tG * bm;
    for (int i = 0; i < 3; ++i) {
      const double dMv = -muB * uG[i] * bm;
      D[5 * (1 + i)] += dMv * dUdRho[i];
      D[6 * (1 + i)] += dMv * dUdRhoU;
      D[21 + i] += dEvdT * dTdRhoU[i];
    }
    D[20] += dEvdT * (-1.0 / (Cv * rhoI) * (EI - magU2));
    D[24] += dEvdT * dTdRhoE;
  }
  for (int k = 0; k < 25; ++k) bjac[k * B + b] = D[k];
}

// Cyclic faces: the coupled part of insertBlock (diag += 0.5|S| A_L, the
// interface block 0.5|S| A_R), of -div(w, u_MRF |S|) (diag -= phi w, the
// interface -= phi (1-w)) and of insertDissipationBlock (diag += 0.5|S|
// lambda, the interface -= the same) -- no boundary-condition terms on a
// coupled patch (blockFvMatrix.C:211-326, convectiveFluxScheme.C:219-232).
// The interface block multiplies the partner's unknowns with their momentum
// rotated into this side's frame (Amul: patchNeighbourField of psi,
// blockFvMatrix.C:386-407), so the stored block is U_f diag(1, R, 1).
// vsf2: the LF viscous coefficient; vj with W, prim and the boundary state:
// the non-LF viscous laplacians, whose interface takes the fields at the
// coupled patch value and whose diagonal takes them at the owner cell
// (blockFvOperatorsTemplates.C:428-448).
template <typename T>
__global__ void k_jac_cyclic(DevMesh m, double gamma, const double* __restrict__ cfrec,
                             const double* __restrict__ flam, double* __restrict__ bjac, T* __restrict__ cblk,
                             const double* __restrict__ vsf2, const double* __restrict__ vj,
                             const double* __restrict__ W, const double* __restrict__ prim,
                             const double* __restrict__ pB, const double* __restrict__ TB,
                             const double* __restrict__ UBv, double Rgas, double Cv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.ncyc) return;
  const int B = m.B, nc = m.ncyc;
  const int b = m.cyc_face[i];
  const double* R = m.patches[m.bpatch[b]].R;
  const double n[3] = {m.bnf[b], m.bnf[B + b], m.bnf[2 * B + b]};
  const double UL[3] = {cfrec[i], cfrec[nc + i], cfrec[2 * nc + i]};
  const double UR[3] = {cfrec[3 * nc + i], cfrec[4 * nc + i], cfrec[5 * nc + i]};
  EulerJ<double> AL, AR;
  AL.init(gamma, UL, cfrec[6 * nc + i], n);
  AR.init(gamma, UR, cfrec[7 * nc + i], n);
  const double magS = m.bmagSf[b];
  const double hs = 0.5 * magS;
  const double d = 0.5 * magS * flam[m.F + b];
  double phm = 0.0;
  if (m.mrfU) phm = m.mrfU[m.F + b] * magS;
  const double wb = m.bw[b];
  // viscous LF: the coupled laplacian's diagonal and interface (viscousFluxScheme.C:234-247)
  const double sv = vsf2 ? vsf2[m.F + b] : 0.0;
  double D[25], U[25];
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      const int k = 5 * r + c;
      double dg = -(-0.5 * magS * AL.entry(r, c));
      double up = hs * AR.entry(r, c);
      if (r == c) {
        dg -= phm * wb;
        up -= phm * (1.0 - wb);
        dg += d;
        up -= d;
        dg += sv;
        up -= sv;
      }
      D[k] = dg;
      U[k] = up;
    }
  if (vj) {
    const int N = m.N, FB = m.F + B, o = m.bcell[b];
    const double mg = vj[m.F + b], ag = vj[FB + m.F + b];
    ViscLapField fo, fb;
    const double Uo[3] = {prim[2 * N + o], prim[3 * N + o], prim[4 * N + o]};
    const double Ub[3] = {UBv[b], UBv[B + b], UBv[2 * B + b]};
    fo.init(W[5 * o], Uo, prim[N + o], Cv);
    fb.init((1.0 / (Rgas * TB[b])) * pB[b], Ub, TB[b], Cv);
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        D[5 * r + c] += fo.entry(r, c, mg, ag);
        U[5 * r + c] -= fb.entry(r, c, mg, ag);
      }
  }
#pragma unroll
  for (int k = 0; k < 25; ++k) bjac[k * B + b] = D[k];
  T* out = cblk + (size_t)i * 25;
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    out[5 * r] = T(U[5 * r]);
    out[5 * r + 4] = T(U[5 * r + 4]);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      out[5 * r + 1 + c] =
          T(U[5 * r + 1] * R[c] + U[5 * r + 2] * R[3 + c] + U[5 * r + 3] * R[6 + c]);
  }
}

// Row assembly.  T = block storage/compute type; VJ: the non-LF viscous
// laplacians (vj, W, prim, Cv used only then).
template <typename T, bool VJ>
__global__ void __launch_bounds__(128) k_jac_rows(DevMesh m, double gamma, const double* __restrict__ frec,
                                                  const double* __restrict__ flam, const double* __restrict__ bjac,
                                                  const double* __restrict__ ddtCoeff, T* __restrict__ blk,
                                                  T* __restrict__ dg, T* __restrict__ rD, int* __restrict__ status,
                                                  const double* __restrict__ vsf2, const double* __restrict__ vj,
                                                  const double* __restrict__ W, const double* __restrict__ prim,
                                                  double Cv) {
  // vsf2 (viscous cases, LaxFriedrichJacobian): LF viscous coefficient
  // 0.5 lambda_v |S| deltaCoeffs, subtracted from the off-diagonal and added
  // to the diagonal entries (viscousFluxScheme.C:234-247); nullptr otherwise.
  // VJ: each face adds the five laplacians at this cell to the diagonal and
  // minus those at the other cell to the off-diagonal block
  // (viscousFluxScheme.C:259-267, blockFvOperatorsTemplates.C:386-420).
  // Off-diagonal slots are stored factored (blocks.cuh): s = +-0.5|S| n,
  // the side's (U, E) and c0 = the identity multiple; with VJ the slot's two
  // laplacian coefficients go to vjslot and this cell's five fields to vjcell.
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int F = m.F, B = m.B;
  ViscLapField vfc;
  if constexpr (VJ) {
    const int N = m.N;
    const double Uc[3] = {prim[2 * N + c], prim[3 * N + c], prim[4 * N + c]};
    vfc.init(W[5 * c], Uc, prim[N + c], Cv);
    T* vc = (T*)m.vjcell;
    for (int k = 0; k < 3; ++k) vc[k * N + c] = T(vfc.mUr[k]);
    vc[3 * N + c] = T(vfc.ir);
    vc[4 * N + c] = T(vfc.eR);
  }
  const int s = c >> 5, lane = c & 31;
  T diag[25];
#pragma unroll
  for (int k = 0; k < 25; ++k) diag[k] = T(0);
  const T g = T(gamma);
  const int base = m.slot_base[s];
  const int width = m.slot_base[s + 1] - base;
  const int ns = m.nslot[c];
  for (int t = 0; t < width; ++t) {
    const int idx = (base + t) * 32 + lane;
    constexpr int SW = SlotBlock<T>::W;  // 8 factored (FP32) or 25 full (FP64) words
    T* out = blk + (size_t)(base + t) * SW * 32 + lane;
    T* vout = VJ ? (T*)m.vjslot + (size_t)(base + t) * 2 * 32 + lane : nullptr;
    if (t >= ns) {
#pragma unroll
      for (int k = 0; k < SW; ++k) out[k * 32] = T(0);
      if constexpr (VJ) vout[0] = vout[32] = T(0);
      continue;
    }
    const int code = m.sface[idx];
    const bool isOwn = code >= 0;
    const int f = isOwn ? code : ~code;
    const T nn[3] = {T(m.nf[f]), T(m.nf[F + f]), T(m.nf[2 * F + f])};
    const T UL[3] = {T(frec[f]), T(frec[F + f]), T(frec[2 * F + f])};
    const T UR[3] = {T(frec[3 * F + f]), T(frec[4 * F + f]), T(frec[5 * F + f])};
    // the diagonal takes minus the other orientation's block: -lower_f in
    // the owner's row (A(W_L), -0.5|S|), -upper_f in the neighbour's row
    EulerJ<T> Ad;
    Ad.init(g, isOwn ? UL : UR, T(frec[(isOwn ? 6 : 7) * F + f]), nn);
    const T magS = T(m.magSf[f]);
    const T hs = T(0.5) * magS;
    const T mhs = T(-0.5) * magS;
    const T d = T(0.5) * magS * T(flam[f]);
    const T sv = vsf2 ? T(vsf2[f]) : T(0);
    // MRF: -div(w, u_MRF |S|) on the diagonal entries (convectiveFluxScheme.C:477-481,
    // blockFvOperatorsTemplates.C:148-197): upper -= phi (1-w), lower += phi w,
    // and the matching negative column sums on the diagonal
    double mg = 0.0, ag = 0.0;
    if constexpr (VJ) {
      mg = vj[f];
      ag = vj[F + B + f];
      vout[0] = T(mg);
      vout[32] = T(ag);
    }
    T moff = T(0), mdg = T(0);
    if (m.mrfU) {
      const double phm = m.mrfU[f] * m.magSf[f], wf = m.w[f];
      moff = isOwn ? T(-(phm * (1.0 - wf))) : T(phm * wf);
      mdg = isOwn ? T(-(phm * wf)) : T(phm * (1.0 - wf));
    }
    // row own: this slot is upper_f = A(U_R, 0.5|S| n) + c0 I and the
    // diagonal gains -lower_f; row nei: lower_f = A(U_L, -0.5|S| n) + c0 I
    const T sg = isOwn ? hs : mhs;
    const T* Us = isOwn ? UR : UL;
    const T Es = T(frec[(isOwn ? 7 : 6) * F + f]);
    if constexpr (SW == 8) {
      out[0] = sg * nn[0];
      out[32] = sg * nn[1];
      out[64] = sg * nn[2];
      out[96] = Us[0];
      out[128] = Us[1];
      out[160] = Us[2];
      out[192] = Es;
      out[224] = ((moff - d) - sv);
    } else {
      EulerJ<T> As;
      As.init(g, Us, Es, nn);
#pragma unroll
      for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          T off = sg * As.entry(i, j);
          if (i == j) {
            off += moff;
            off -= d;
            off -= sv;
          }
          out[(5 * i + j) * 32] = off;
        }
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const int k = 5 * i + j;
        diag[k] -= (isOwn ? mhs : hs) * Ad.entry(i, j);
        if (i == j) {
          diag[k] += mdg;
          diag[k] += d;
          diag[k] += sv;
        }
        if constexpr (VJ) diag[k] += T(vfc.entry(i, j, mg, ag));
      }
    }
  }
  const int b0 = m.bptr[c], b1 = m.bptr[c + 1];
  for (int e = b0; e < b1; ++e) {
    const int b = m.bface[e];
#pragma unroll
    for (int k = 0; k < 25; ++k) diag[k] += T(bjac[k * B + b]);
  }
  const T dc = T(ddtCoeff[c] * m.V[c]);
#pragma unroll
  for (int q = 0; q < 5; ++q) diag[6 * q] += dc;
  if (m.mrfOm) {
    // MRF source block: skew(omega) V on the momentum diagonal block
    // (convectiveFluxScheme.C:131-137)
    const int N = m.N;
    const double Vc = m.V[c];
    const double ox = m.mrfOm[c] * Vc, oy = m.mrfOm[N + c] * Vc, oz = m.mrfOm[2 * N + c] * Vc;
    diag[5 * 1 + 2] -= T(oz);
    diag[5 * 1 + 3] += T(oy);
    diag[5 * 2 + 1] += T(oz);
    diag[5 * 2 + 3] -= T(ox);
    diag[5 * 3 + 1] -= T(oy);
    diag[5 * 3 + 2] += T(ox);
  }
  if (m.nInst > 1 && hb_in_zone(m, c)) {
    // Harmonic Balance diagonal V D_JJ on every equation, in the HB zone
    // (HBZone.C:435-518: Cartesian, cylCoords or not)
    const int J = c / m.Nc;
    const T hd = T(m.V[c] * m.Dhb[J * m.nInst + J]);
#pragma unroll
    for (int q = 0; q < 5; ++q) diag[6 * q] += hd;
  }
  T* dout = dg + (size_t)s * 25 * 32 + lane;
#pragma unroll
  for (int k = 0; k < 25; ++k) dout[k * 32] = diag[k];
  // LU-SGS scalar diagonal: rD = 1/max over the five diagonal entries
  double r = GREAT;
  const int order[5] = {0, 24, 6, 12, 18};
#pragma unroll
  for (int q = 0; q < 5; ++q) r = 1.0 / fmax(1.0 / r, fabs((double)diag[order[q]]));
  if (!(r >= VSMALL)) atomicOr(status, 1);
  rD[c] = T(r);
}

// 5x5 block inverses for the Jacobi preconditioner (Jacobi.C:55-135 with
// JacobiSmoother::calcInvDiag); Gauss-Jordan with partial pivoting.
template <typename T>
__global__ void k_jacobi_inverse(int N, const T* __restrict__ dg, T* __restrict__ inv, int* __restrict__ status) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const int s = c >> 5, lane = c & 31;
  double a[5][10];
  const T* src = dg + (size_t)s * 25 * 32 + lane;
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      a[i][j] = (double)src[(5 * i + j) * 32];
      a[i][5 + j] = i == j ? 1.0 : 0.0;
    }
  for (int k = 0; k < 5; ++k) {
    int p = k;
    double mx = fabs(a[k][k]);
    for (int i = k + 1; i < 5; ++i)
      if (fabs(a[i][k]) > mx) {
        mx = fabs(a[i][k]);
        p = i;
      }
    if (mx == 0.0) {
      atomicOr(status, 1);
      return;
    }
    if (p != k)
      for (int j = 0; j < 10; ++j) {
        double t = a[k][j];
        a[k][j] = a[p][j];
        a[p][j] = t;
      }
    const double piv = a[k][k];
    for (int j = 0; j < 10; ++j) a[k][j] /= piv;
    for (int i = 0; i < 5; ++i) {
      if (i == k) continue;
      const double fct = a[i][k];
      for (int j = 0; j < 10; ++j) a[i][j] -= fct * a[k][j];
    }
  }
  T* dst = inv + (size_t)s * 25 * 32 + lane;
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) dst[(5 * i + j) * 32] = T(a[i][5 + j]);
}

// every slot's 25 entries (A(U, E, s) + c0 I minus the non-LF viscous part)
template <typename TB>
__global__ void k_expand_slots(DevMesh m, const TB* __restrict__ blk, double* __restrict__ out) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;  // slot * 32 + lane
  if (i >= (long)m.nslots * 32) return;
  const size_t slot = (size_t)(i / 32);
  const int lane = (int)(i % 32);
  SlotBlock<TB> Bk;
  Bk.load(blk, slot, lane);
  const int col = m.scol[i];
  const bool vj = m.vjslot && col >= 0 && col < m.N;  // padding slots have no column
  for (int k = 0; k < 25; ++k) {
    double e = Bk.entry(m.gamma, k / 5, k % 5);
    if (vj) e -= vj_entry<TB>(m, slot, lane, col, k / 5, k % 5);
    out[(slot * 25 + k) * 32 + lane] = e;
  }
}

void launch_expand_slots(Handle& h, double* out) {
  const long n = (long)h.m.nslots * 32;
  if (h.jacPrecision == ICS_PREC_MIXED)
    k_expand_slots<float><<<grid_for(n, 128), 128, 0, h.stream>>>(h.m, (const float*)h.blk, out);
  else
    k_expand_slots<double><<<grid_for(n, 128), 128, 0, h.stream>>>(h.m, (const double*)h.blk, out);
  ICS_CUDA(cudaGetLastError());
}

void launch_jacobian(Handle& h) {
  // viscous Jacobian: LF coefficient (vsf2) or the non-LF laplacians (vj)
  const bool visc = h.cfg.c.viscous != 0, lf = h.cfg.c.viscous_lf_jacobian != 0;
  const double* vsf2 = visc && lf ? h.vsf2 : nullptr;
  const double* vj = visc && !lf ? h.vjac : nullptr;
  // the non-LF viscous parts of the off-diagonal blocks (blocks.cuh)
  if (vj) {
    if (!h.vjslotbuf) {  // FP64-sized: serves both precisions
      ICS_CUDA(cudaMalloc(&h.vjslotbuf, (size_t)h.m.nslots * 2 * 32 * sizeof(double)));
      ICS_CUDA(cudaMalloc(&h.vjcellbuf, 5ull * h.m.N * sizeof(double)));
    }
    h.m.vjslot = h.vjslotbuf;
    h.m.vjcell = h.vjcellbuf;
  } else {
    h.m.vjslot = h.m.vjcell = nullptr;
  }
  if (h.m.B > 0)
    ICS_LAUNCH(h, ICS_K_JAC_BOUNDARY, k_jac_boundary<<<grid_for(h.m.B, 128), 128, 0, h.stream>>>(h.m, h.cfg.c.R, h.cfg.Cv, h.cfg.gamma, h.W, h.prim,
                                                                h.pB, h.TB, h.UB, h.phiB, h.flam, h.bjac, vj));
  int* status = &h.ks->status;
  if (h.m.ncyc > 0) {
    if (prec(h) == ICS_PREC_MIXED)
      ICS_LAUNCH(h, ICS_K_JAC_BOUNDARY, k_jac_cyclic<float><<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(
                                            h.m, h.cfg.gamma, h.cfrec, h.flam, h.bjac, (float*)h.cblk, vsf2, vj,
                                            h.W, h.prim, h.pB, h.TB, h.UB, h.cfg.c.R, h.cfg.Cv));
    else
      ICS_LAUNCH(h, ICS_K_JAC_BOUNDARY, k_jac_cyclic<double><<<grid_for(h.m.ncyc, 128), 128, 0, h.stream>>>(
                                            h.m, h.cfg.gamma, h.cfrec, h.flam, h.bjac, (double*)h.cblk, vsf2, vj,
                                            h.W, h.prim, h.pB, h.TB, h.UB, h.cfg.c.R, h.cfg.Cv));
  }
  if (prec(h) == ICS_PREC_MIXED) {
    if (vj)
      ICS_LAUNCH(h, ICS_K_JAC_ROWS, k_jac_rows<float, true><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(
                                        h.m, h.cfg.gamma, h.frec, h.flam, h.bjac, h.ddtCoeff, (float*)h.blk,
                                        (float*)h.dg, (float*)h.rD, status, vsf2, vj, h.W, h.prim, h.cfg.Cv));
    else
      ICS_LAUNCH(h, ICS_K_JAC_ROWS, k_jac_rows<float, false><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(
                                        h.m, h.cfg.gamma, h.frec, h.flam, h.bjac, h.ddtCoeff, (float*)h.blk,
                                        (float*)h.dg, (float*)h.rD, status, vsf2, nullptr, nullptr, nullptr, 0.0));
    if (h.cfg.c.preconditioner == ICS_PC_JACOBI || h.cfg.c.solver == ICS_SOLVER_SMOOTH)
      ICS_LAUNCH(h, ICS_K_JACOBI_INV, k_jacobi_inverse<float><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m.N, (float*)h.dg, (float*)h.dginv,
                                                                          status));
  } else {
    if (vj)
      ICS_LAUNCH(h, ICS_K_JAC_ROWS, k_jac_rows<double, true><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(
                                        h.m, h.cfg.gamma, h.frec, h.flam, h.bjac, h.ddtCoeff, (double*)h.blk,
                                        (double*)h.dg, (double*)h.rD, status, vsf2, vj, h.W, h.prim, h.cfg.Cv));
    else
      ICS_LAUNCH(h, ICS_K_JAC_ROWS, k_jac_rows<double, false><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(
                                        h.m, h.cfg.gamma, h.frec, h.flam, h.bjac, h.ddtCoeff, (double*)h.blk,
                                        (double*)h.dg, (double*)h.rD, status, vsf2, nullptr, nullptr, nullptr, 0.0));
    if (h.cfg.c.preconditioner == ICS_PC_JACOBI || h.cfg.c.solver == ICS_SOLVER_SMOOTH)
      ICS_LAUNCH(h, ICS_K_JACOBI_INV, k_jacobi_inverse<double><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m.N, (double*)h.dg, (double*)h.dginv,
                                                                           status));
  }
  ICS_CUDA(cudaGetLastError());
  h.jacPrecision = prec(h);
}

}  // namespace ics
