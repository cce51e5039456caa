// icsref - CPU FP64 oracle for the implicit coupled pseudo-time iteration.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference arm of bench.py may load this library, and only as
// the checker or the timed CPU baseline - never as part of the product path.
//
// A sequential restatement, written field-by-field in the style of the
// reference, of ICSFoam's dbnsFoam pseudo-time iteration:
//   fluxes          ausmPlusUpFluxScheme.C:73-299, hllcFluxScheme.C:70-240,
//                   roeFluxScheme.C:41-409, cellFaceFunctions.H:491-661
//   residual        applications/solvers/dbnsFoam/residualsUpdate.H:1-83
//   local dtau, SER setCoAndDeltaT.H:1-173
//   Jacobian        convectiveFluxScheme.C:47-546, blockFvMatrix.C:211-326
//   linear algebra  blockFvMatrix.C:329-601, coupledMatrix.C:66-385,
//                   coupledMatrixSolver.C:99-221, gmres.C:44-1107,
//                   lusgs.C:50-385, Jacobi.C:55-135, JacobiSmoother.C:42-205
//   update          boundLocalTimeStep.H:1-97, updateFields.H:1-105
//   control         pseudotimeControl.C:42-241, pseudotimeControlI.H:42-69
//   dual time       dualTimeDdtScheme.C:111-185
// The OpenFOAM v2112 pieces these call (limitedScheme/linearUpwind
// interpolation, Gauss gradients, cellLimited gradient limiting, Euler and
// backward ddt, boundary conditions, perfect-gas thermo, LUscalarMatrix) are
// restated from their documented mathematics; OpenFOAM itself is absent.
//
// Parity against the reference binary is unpinned: the reference has no
// tests or golden data and cannot be built without OpenFOAM.  The oracle is
// pinned instead by analytic known-answer tests (tests/test_oracle_*.py).
//
// Built with -ffp-contract=off so x86 and Arm produce identical bits.

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "../include/icsfoam_gb300.h"

namespace {

constexpr double SMALL = 1e-15;
constexpr double VSMALL = 1e-300;
constexpr double ROOTVSMALL = 1e-150;
constexpr double GREAT = 1e15;
constexpr double VGREAT = 1e300;

struct V3 {
  double x = 0, y = 0, z = 0;
  V3() = default;
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(double s, const V3& a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(const V3& a, double s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(const V3& a, double s) { return V3(a.x / s, a.y / s, a.z / s); }
inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double magSqr(const V3& a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline double mag(const V3& a) { return std::sqrt(magSqr(a)); }
inline double pos0(double s) { return s >= 0 ? 1.0 : 0.0; }
inline double neg(double s) { return s < 0 ? 1.0 : 0.0; }
inline double sgn(double s) { return s >= 0 ? 1.0 : -1.0; }
inline double sqr(double s) { return s * s; }

// 3x3 tensor, row-major T[i][j]
struct T33 {
  double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
};
inline T33 outer(const V3& u, const V3& v) {
  T33 t;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t.a[i][j] = u[i] * v[j];
  return t;
}

// 5x5 block in variable order (rho, rhoUx, rhoUy, rhoUz, rhoE)
struct B5 {
  double a[25];
  B5() { std::memset(a, 0, sizeof(a)); }
  double& operator()(int i, int j) { return a[i * 5 + j]; }
  double operator()(int i, int j) const { return a[i * 5 + j]; }
};

struct Patch {
  int kind, is_wall;
  double p, T, U[3], p0, T0;
  double R[9];  // cyclic: partner-side vectors into this patch's frame
};

struct Case {
  // mesh
  int N = 0, F = 0, B = 0;
  std::vector<int> own, nei, bcell, bpatch;
  std::vector<V3> Sf, Cf, C, bSf, bCf;
  std::vector<double> magSf, bmagSf, w, dc, nodc, V, bdc;
  std::vector<Patch> patches;
  int solD[3] = {1, 1, 1};
  std::vector<std::vector<int>> cellFaces;  // OpenFOAM cells(): owner faces then neighbour faces
  ics_config cfg{};
  double Cv = 0, gamma = 0;

  // state (internal)
  std::vector<double> rho, rhoE, p, T, e;
  std::vector<V3> rhoU, U;
  // boundary values
  std::vector<double> pB, TB, phiB;
  std::vector<V3> UB;
  // old time levels
  std::vector<double> rho0, rhoE0, rho00, rhoE00;
  std::vector<V3> rhoU0, rhoU00;
  int timeIndex = 0;  // number of begun physical time steps
  // pseudo time
  std::vector<double> pseudoCo, rPseudoDeltaT, ddtCoeff;
  // LF viscous Jacobian coefficient per internal face (from the last residual)
  std::vector<double> viscSf2;
  // laplacian coefficients of the non-LF viscous Jacobian (F+B): internal and
  // coupled faces (mu_f |S|) deltaCoeffs and (alphaEff_f |S|) deltaCoeffs,
  // physical boundary faces the patch values mu_b and alphaEff_b
  std::vector<double> viscMuG, viscAlG;
  // fluxes of the last calcFlux (F+B)
  std::vector<double> phi, phiE;
  std::vector<V3> phiU;
  double lastRhoL2 = 0;
  // matrix: LDU of 5x5 blocks + source
  std::vector<B5> diag, lower, upper;
  std::vector<double> src;  // N*5
  bool haveMatrix = false;
  // previous-iteration state and increment
  std::vector<double> Wprev, dW;  // N*5
  bool haveIncrement = false;
  // Harmonic Balance: nInst stacked instances of Nc cells, operator Dhb
  int nInst = 1, Nc = 0;
  std::vector<double> Dhb;
  // HB zone (HBZone cellZone; empty: every cell) and cylCoords about axis / origin
  std::vector<unsigned char> hbZone;
  bool hbCyl = false;
  V3 hbAxis = V3(0, 0, 1), hbOrigin = V3();
  // residual bookkeeping (setCoAndDeltaT.H, pseudotimeControl), one entry per
  // equation and instance: [5*J + k], k = rho, rhoUx, rhoUy, rhoUz, rhoE
  bool initResValid = false, prevResValid = false;
  std::vector<double> initRes, prevRes;
  // pseudotimeControl state, one per instance (the HB solver keeps one
  // control per sub-time mesh and loops while any of them is not finished)
  struct Control {
    int corr = 0;
    bool converged = false, firstIteration = true;
    double residuals[5] = {0, 0, 0, 0, 0}, initResiduals[5] = {0, 0, 0, 0, 0};
  };
  std::vector<Control> ctl = std::vector<Control>(1);
  // passive scalar transport (dbnsFoam calculateScalarTransport.H): s and the
  // transported rhoS (with old time levels), boundary values, per-patch BC
  bool scalarOn = false;
  double Ds = 0;
  int reconS = ICS_RECON_UPWIND;
  std::vector<double> s, sB, rhoS, rhoS0, rhoS00;
  std::vector<int> sFixed;
  std::vector<double> sValue;
  // coupled (cyclic) boundary faces: partner cell (-1 elsewhere), linear
  // weight, delta (partner centre seen from this side minus C), partner-side
  // displacement Cf - C - delta, nonOrthDeltaCoeffs, and the interface
  // blocks of the last Jacobian (blockFvMatrix interfacesUpper)
  bool hasCyc = false;
  // phase-lag cyclic patches of Harmonic Balance handles (phaseLagCyclic):
  // per patch 0 = plain cyclic, 1 = phase lag, 2 = phase lag with the velocity
  // combined in cylindrical components; the n x n operator Re(E^-1 M E) of each
  std::vector<int> plagMode;
  std::vector<double> plagP;
  std::vector<int> bpartner;
  std::vector<double> bw, bnodc;
  std::vector<V3> bdelta, bnbrd;
  std::vector<B5> iface;
  // moving reference frames (dbnsFoam outerLoop.H:6-21): frame velocity . n
  // per internal then boundary face, rotation vector per cell, frame velocity
  // of the boundary faces that correctBoundaryVelocity assigns
  bool mrfOn = false;
  int mrfEvery = 0;
  std::vector<double> mrfU;
  std::vector<V3> mrfOm, mrfBU;
  std::vector<int> mrfBIn;
  std::string err;
};

// cyclic boundary face b, and R v with the rotation of its patch
inline bool isCyc(const Case& c, int b) { return c.hasCyc && c.bpartner[b] >= 0; }
inline V3 rotP(const Case& c, int b, const V3& v) {
  const double* R = c.patches[c.bpatch[b]].R;
  return V3(R[0] * v.x + R[1] * v.y + R[2] * v.z, R[3] * v.x + R[4] * v.y + R[5] * v.z,
            R[6] * v.x + R[7] * v.y + R[8] * v.z);
}

// a vol field: internal values + boundary-face values
struct VolS {
  std::vector<double> in, bf;
  std::vector<double> nb;  // phase-lagged neighbour values of the phase-lag cyclic faces (or empty)
};

// phase-lag cyclic face b (phaseLagCyclicFvPatchField::patchNeighbourField,
// phaseLagCyclicFvPatchFields.C): the neighbour value of instance J of a
// phase-lagged field is sum_K P_JK f_K(partner), P = Re(E^-1 M(+-IBPA) E)
inline bool isPlag(const Case& c, int b) {
  return isCyc(c, b) && !c.plagMode.empty() && c.plagMode[c.bpatch[b]] > 0;
}
template <typename Fn>
double plagSum(const Case& c, int b, Fn f) {
  const int n = c.nInst, pc = c.bpartner[b], J = pc / c.Nc, cl = pc % c.Nc;
  const double* P = &c.plagP[((size_t)c.bpatch[b] * n + J) * n];
  double s = 0;
  for (int K = 0; K < n; ++K) s += P[K] * f(K * c.Nc + cl);
  return s;
}
// the velocity: combined as it is (mode 1) or, with cylindrical coordinates,
// combined and rotated into this side's frame (mode 2)
inline V3 plagVec(const Case& c, int b, const std::vector<V3>& U) {
  V3 v;
  for (int k = 0; k < 3; ++k) v[k] = plagSum(c, b, [&](int q) { return U[q][k]; });
  return c.plagMode[c.bpatch[b]] == 2 ? rotP(c, b, v) : v;
}
// neighbour value of a scalar field on cyclic face b
inline double nbOf(const Case& c, const VolS& f, int b) {
  return (!f.nb.empty() && isPlag(c, b)) ? f.nb[b] : f.in[c.bpartner[b]];
}
template <typename Fn>
void setPlag(const Case& c, VolS& f, Fn cellValue) {
  if (c.plagMode.empty()) return;
  f.nb.assign(c.B, 0.0);
  for (int b = 0; b < c.B; ++b)
    if (isPlag(c, b)) f.nb[b] = plagSum(c, b, cellValue);
}

// MRF face velocity of face fi (internal then boundary), zero without zones
inline double umOf(const Case& c, int fi) { return c.mrfOn ? c.mrfU[fi] : 0.0; }

// HBZone cellZone membership of cell i (every cell without a zone)
inline bool hbInZone(const Case& c, int i) { return c.hbZone.empty() || c.hbZone[i]; }

// radial and circumferential unit vectors of the HB zone's cylindrical frame
// at the centre of cell i (HBZone.C:560-582)
inline void hbFrame(const Case& c, int i, V3& rh, V3& th) {
  V3 r = c.C[i] - c.hbOrigin;
  r = r - c.hbAxis * dot(c.hbAxis, r);
  rh = r / std::sqrt(dot(r, r));
  th = V3(c.hbAxis.y * rh.z - c.hbAxis.z * rh.y, c.hbAxis.z * rh.x - c.hbAxis.x * rh.z,
          c.hbAxis.x * rh.y - c.hbAxis.y * rh.x);
}

// MRFCoupledZone::correctBoundaryVelocity (MRFCoupledZone.C:594-619)
void mrfBoundaryVelocity(Case& c) {
  if (!c.mrfOn) return;
  for (int b = 0; b < c.B; ++b)
    if (c.mrfBIn[b]) c.UB[b] = c.mrfBU[b];
}

// ---------------------------------------------------------------------------
// Thermo: perfectGas + hConst + sensibleInternalEnergy, Tref = 0
// ---------------------------------------------------------------------------
inline double psiOf(const Case& c, double T) { return 1.0 / (c.cfg.R * T); }
inline double heOf(const Case& c, double T) { return c.Cv * T; }

// ---------------------------------------------------------------------------
// Field helpers: a vol field = internal values + boundary-face values
// ---------------------------------------------------------------------------

// Gauss linear gradient (OpenFOAM gaussGrad with linear interpolation)
void gaussGrad(const Case& c, const VolS& f, std::vector<V3>& g) {
  g.assign(c.N, V3());
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    const double sf = c.w[fi] * (f.in[o] - f.in[n]) + f.in[n];
    const V3 Ssf = c.Sf[fi] * sf;
    g[o] = g[o] + Ssf;
    g[n] = g[n] - Ssf;
  }
  for (int b = 0; b < c.B; ++b) {
    const int o = c.bcell[b];
    if (isCyc(c, b)) {  // linear interpolation with the partner (coupled patch)
      const double fn = nbOf(c, f, b);
      g[o] = g[o] + c.bSf[b] * (c.bw[b] * (f.in[o] - fn) + fn);
      continue;
    }
    g[o] = g[o] + c.bSf[b] * f.bf[b];
  }
  for (int i = 0; i < c.N; ++i) g[i] = g[i] / c.V[i];
}

// cellLimited<limiter> Gauss linear 1 (cellLimitedGrad): minmod or Venkatakrishnan
void cellLimitedGrad(const Case& c, const VolS& f, bool venkat, std::vector<V3>& g) {
  gaussGrad(c, f, g);
  std::vector<double> maxV(f.in), minV(f.in);
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    maxV[o] = std::max(maxV[o], f.in[n]);
    minV[o] = std::min(minV[o], f.in[n]);
    maxV[n] = std::max(maxV[n], f.in[o]);
    minV[n] = std::min(minV[n], f.in[o]);
  }
  for (int b = 0; b < c.B; ++b) {
    const int o = c.bcell[b];
    const double v = isCyc(c, b) ? nbOf(c, f, b) : f.bf[b];  // coupled: the neighbour cell
    maxV[o] = std::max(maxV[o], v);
    minV[o] = std::min(minV[o], v);
  }
  for (int i = 0; i < c.N; ++i) {
    maxV[i] -= f.in[i];
    minV[i] -= f.in[i];
  }
  // the coefficient k of "cellLimited<..> Gauss linear k": for k < 1 the
  // bounds widen by (1/k - 1)(max - min) (cellLimitedGrad::calcGrad)
  if (c.cfg.limiter_coeff < 1.0) {
    const double widen = 1.0 / c.cfg.limiter_coeff - 1.0;
    for (int i = 0; i < c.N; ++i) {
      const double d = widen * (maxV[i] - minV[i]);
      maxV[i] += d;
      minV[i] -= d;
    }
  }
  std::vector<double> lim(c.N, 1.0);
  auto limitFace = [&](double& l, double maxD, double minD, double extrap) {
    double r = 1;
    if (extrap > SMALL)
      r = maxD / extrap;
    else if (extrap < -SMALL)
      r = minD / extrap;
    double lr = venkat ? (sqr(r) + 2 * r) / (sqr(r) + r + 2) : std::min(r, 1.0);
    l = std::min(l, lr);
  };
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    limitFace(lim[o], maxV[o], minV[o], dot(c.Cf[fi] - c.C[o], g[o]));
    limitFace(lim[n], maxV[n], minV[n], dot(c.Cf[fi] - c.C[n], g[n]));
  }
  for (int b = 0; b < c.B; ++b) {
    const int o = c.bcell[b];
    limitFace(lim[o], maxV[o], minV[o], dot(c.bCf[b] - c.C[o], g[o]));
  }
  for (int i = 0; i < c.N; ++i) g[i] = g[i] * lim[i];
}

// linear interpolation (internal + boundary values)
void interpLinear(const Case& c, const VolS& f, std::vector<double>& out) {
  out.resize(c.F + c.B);
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    out[fi] = c.w[fi] * (f.in[o] - f.in[n]) + f.in[n];
  }
  for (int b = 0; b < c.B; ++b) {
    if (isCyc(c, b)) {
      const double fn = nbOf(c, f, b);
      out[c.F + b] = c.bw[b] * (f.in[c.bcell[b]] - fn) + fn;
    } else {
      out[c.F + b] = f.bf[b];
    }
  }
}

// fvc::interpolate(vf, dir, "reconstruct(..)") for the configured scheme.
void reconstruct(const Case& c, const VolS& f, double dir, int scheme, std::vector<double>& out) {
  out.resize(c.F + c.B);
  const double wUp = pos0(dir);
  const bool tvd = scheme == ICS_RECON_VANLEER || scheme == ICS_RECON_MINMOD;
  std::vector<V3> g;
  if (tvd)
    gaussGrad(c, f, g);
  else if (scheme != ICS_RECON_UPWIND)
    cellLimitedGrad(c, f, scheme == ICS_RECON_MUSCL_VENKATAKRISHNAN, g);
  // TVD limitedScheme weight of a face with upwind-side gradient gu
  auto tvdValue = [&](double phiP, double phiN, const V3& d, const V3& gu, double cdw) {
    const double gradf = phiN - phiP;
    const double gradcf = dot(d, gu);
    double r;
    if (std::fabs(gradcf) >= 1000 * std::fabs(gradf))
      r = 2 * 1000 * sgn(gradcf) * sgn(gradf) - 1;
    else
      r = 2 * (gradcf / gradf) - 1;
    double lim;
    if (scheme == ICS_RECON_VANLEER)
      lim = (r + std::fabs(r)) / (1 + std::fabs(r));
    else
      lim = std::max(std::min(std::min(r, 1.0), 2.0), 0.0);
    const double wgt = lim * cdw + (1.0 - lim) * wUp;
    return wgt * (phiP - phiN) + phiN;
  };
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    const double phiP = f.in[o], phiN = f.in[n];
    if (scheme == ICS_RECON_UPWIND) {
      out[fi] = wUp * (phiP - phiN) + phiN;
    } else if (tvd) {
      out[fi] = tvdValue(phiP, phiN, c.C[n] - c.C[o], dir > 0 ? g[o] : g[n], c.w[fi]);
    } else {  // MUSCL: linearUpwind + cellLimited gradient
      const int up = dir > 0 ? o : n;
      const double base = wUp * (phiP - phiN) + phiN;
      out[fi] = base + dot(c.Cf[fi] - c.C[up], g[up]);
    }
  }
  for (int b = 0; b < c.B; ++b) {
    out[c.F + b] = f.bf[b];
    if (!isCyc(c, b)) continue;
    // coupled face: this side's cell o and the partner pc; the partner's
    // value as it is (a scalar field), its gradient rotated into this side's
    // frame; the TVD ratio uses delta, linearUpwind extrapolates the partner
    // side along Cf - C - delta (limitedScheme / linearUpwind on coupled patches)
    const int o = c.bcell[b], pc = c.bpartner[b];
    const double phiP = f.in[o], phiN = nbOf(c, f, b);
    if (scheme == ICS_RECON_UPWIND) {
      out[c.F + b] = wUp * (phiP - phiN) + phiN;
      continue;
    }
    const V3 gu = dir > 0 ? g[o] : rotP(c, b, g[pc]);
    if (tvd) {
      out[c.F + b] = tvdValue(phiP, phiN, c.bdelta[b], gu, c.bw[b]);
    } else {
      const double base = wUp * (phiP - phiN) + phiN;
      const V3 d = dir > 0 ? c.bCf[b] - c.C[o] : c.bnbrd[b];
      out[c.F + b] = base + dot(d, gu);
    }
  }
}

// component fields of U (internal + boundary)
VolS Ucmpt(const Case& c, int k) {
  VolS f;
  f.in.resize(c.N);
  f.bf.resize(c.B);
  for (int i = 0; i < c.N; ++i) f.in[i] = c.U[i][k];
  for (int b = 0; b < c.B; ++b) f.bf[b] = c.UB[b][k];
  if (!c.plagMode.empty()) {  // "U.component(k)"
    f.nb.assign(c.B, 0.0);
    for (int b = 0; b < c.B; ++b)
      if (isPlag(c, b)) f.nb[b] = plagVec(c, b, c.U)[k];
  }
  return f;
}

void reconstructU(const Case& c, double dir, std::vector<V3>& out) {
  out.assign(c.F + c.B, V3());
  std::vector<double> tmp;
  for (int k = 0; k < 3; ++k) {
    reconstruct(c, Ucmpt(c, k), dir, c.cfg.recon_U, tmp);
    for (int fi = 0; fi < c.F + c.B; ++fi) out[fi][k] = tmp[fi];
  }
}

inline const V3& SfOf(const Case& c, int fi) { return fi < c.F ? c.Sf[fi] : c.bSf[fi - c.F]; }
inline double magSfOf(const Case& c, int fi) { return fi < c.F ? c.magSf[fi] : c.bmagSf[fi - c.F]; }

// E = he(p,T) + 0.5|U|^2 and boundary values
VolS fieldE(const Case& c) {
  VolS E;
  E.in.resize(c.N);
  E.bf.resize(c.B);
  for (int i = 0; i < c.N; ++i) E.in[i] = heOf(c, c.T[i]) + 0.5 * magSqr(c.U[i]);
  for (int b = 0; b < c.B; ++b) E.bf[b] = heOf(c, c.TB[b]) + 0.5 * magSqr(c.UB[b]);
  setPlag(c, E, [&](int q) { return heOf(c, c.T[q]) + 0.5 * magSqr(c.U[q]); });
  return E;
}
double rhoBof(const Case& c, int b) { return psiOf(c, c.TB[b]) * c.pB[b]; }

VolS fieldH(const Case& c, const VolS& E) {
  VolS H;
  H.in.resize(c.N);
  H.bf.resize(c.B);
  for (int i = 0; i < c.N; ++i) H.in[i] = std::max(E.in[i], SMALL) + std::max(c.p[i] / c.rho[i], SMALL);
  for (int b = 0; b < c.B; ++b) H.bf[b] = std::max(E.bf[b], SMALL) + std::max(c.pB[b] / rhoBof(c, b), SMALL);
  setPlag(c, H, [&](int q) { return heOf(c, c.T[q]) + 0.5 * magSqr(c.U[q]) + c.p[q] / c.rho[q]; });
  return H;
}
VolS fieldRho(const Case& c) {
  VolS r;
  r.in = c.rho;
  r.bf.resize(c.B);
  for (int b = 0; b < c.B; ++b) r.bf[b] = rhoBof(c, b);
  setPlag(c, r, [&](int q) { return c.rho[q]; });
  return r;
}
VolS fieldP(const Case& c) {
  VolS r;
  r.in = c.p;
  r.bf = c.pB;
  setPlag(c, r, [&](int q) { return c.p[q]; });
  return r;
}
// the phase-lagged neighbour of a sound-speed field is sqrt(gamma/psi) of the
// instances ("c" and "sqrt((gamma|thermo:psi))" alike)
void setPlagC(const Case& c, VolS& f) { setPlag(c, f, [&](int q) { return std::sqrt(c.gamma / psiOf(c, c.T[q])); }); }

// ---------------------------------------------------------------------------
// Flux schemes
// ---------------------------------------------------------------------------
void calcFluxAUSM(Case& c) {
  const int NF = c.F + c.B;
  std::vector<V3> U_L, U_R;
  reconstructU(c, +1, U_L);
  reconstructU(c, -1, U_R);
  std::vector<double> un_L(NF), un_R(NF);
  for (int fi = 0; fi < NF; ++fi) {
    un_L[fi] = dot(U_L[fi], SfOf(c, fi)) / magSfOf(c, fi);
    un_R[fi] = dot(U_R[fi], SfOf(c, fi)) / magSfOf(c, fi);
    un_L[fi] -= umOf(c, fi);  // MRF face velocity (ausmPlusUpFluxScheme.C:101-102)
    un_R[fi] -= umOf(c, fi);
  }
  VolS E = fieldE(c);
  VolS H = fieldH(c, E);
  VolS cs;
  cs.in.resize(c.N);
  cs.bf.resize(c.B);
  const double g = c.gamma;
  for (int i = 0; i < c.N; ++i) cs.in[i] = std::sqrt(2.0 * (g - 1.0) / (g + 1.0) * H.in[i]);
  for (int b = 0; b < c.B; ++b) cs.bf[b] = std::sqrt(2.0 * (g - 1.0) / (g + 1.0) * H.bf[b]);
  setPlagC(c, cs);
  std::vector<double> c_L, c_R;
  reconstruct(c, cs, +1, c.cfg.recon_T, c_L);
  reconstruct(c, cs, -1, c.cfg.recon_T, c_R);
  std::vector<double> c_face(NF);
  for (int fi = 0; fi < NF; ++fi) {
    const double cl = sqr(c_L[fi]) / std::max(c_L[fi], un_L[fi]);
    const double cr = sqr(c_R[fi]) / std::max(c_R[fi], -un_R[fi]);
    c_face[fi] = std::min(cl, cr);
  }
  std::vector<double> p_L, p_R, rho_L, rho_R, H_L, H_R;
  VolS P = fieldP(c), RHO = fieldRho(c);
  reconstruct(c, P, +1, c.cfg.recon_rho, p_L);
  reconstruct(c, P, -1, c.cfg.recon_rho, p_R);
  reconstruct(c, RHO, +1, c.cfg.recon_rho, rho_L);
  reconstruct(c, RHO, -1, c.cfg.recon_rho, rho_R);
  reconstruct(c, H, +1, c.cfg.recon_T, H_L);
  reconstruct(c, H, -1, c.cfg.recon_T, H_R);
  for (int fi = 0; fi < NF; ++fi) {
    const double cf = c_face[fi];
    const double ML = un_L[fi] / cf;
    double Mplus, pplus;
    if (std::fabs(ML) < 1.0) {
      const double ML2p = 0.25 * sqr(ML + 1);
      const double ML2m = -0.25 * sqr(ML - 1);
      Mplus = ML2p * (1 - 2 * ML2m);
      pplus = ML2p * (2 - ML - 3 * ML * ML2m);
    } else {
      Mplus = std::max(ML, 0.0);
      pplus = ML > 0 ? 1.0 : 0.0;
    }
    const double MR = un_R[fi] / cf;
    double Mminus, pminus;
    if (std::fabs(MR) < 1.0) {
      const double MR2m = -0.25 * sqr(MR - 1);
      const double MR2p = 0.25 * sqr(MR + 1);
      Mminus = MR2m * (1 + 2 * MR2p);
      pminus = MR2m * (-2 - MR + 3 * MR * MR2p);
    } else {
      Mminus = std::min(MR, 0.0);
      pminus = MR < 0 ? 1.0 : 0.0;
    }
    double M12 = Mplus + Mminus;
    double p12 = pplus * p_L[fi] + pminus * p_R[fi];
    const double Mmean = 0.5 * (sqr(un_L[fi]) + sqr(un_R[fi])) / sqr(cf);
    const double MDiff =
        -0.25 * std::max((1.0 - Mmean), 0.0) * (p_R[fi] - p_L[fi]) / (0.5 * (rho_L[fi] + rho_R[fi]) * sqr(cf));
    if ((M12 > 0.0 && M12 + MDiff <= 0.0) || (M12 < 0.0 && M12 + MDiff >= 0.0))
      M12 += 0.2 * MDiff;
    else
      M12 += MDiff;
    if (c.cfg.low_mach_ausm) {
      const double pDiff = -0.25 * pplus * pminus * (rho_L[fi] + rho_R[fi]) * cf * (un_R[fi] - un_L[fi]);
      p12 += pDiff;
    }
    const bool left = M12 >= 0;
    const V3 Uf = left ? U_L[fi] : U_R[fi];
    const double rhoa = M12 * cf * (left ? rho_L[fi] : rho_R[fi]);
    const V3 rhoaU = rhoa * Uf;
    const double rhoah = rhoa * (left ? H_L[fi] : H_R[fi]);
    const double ms = magSfOf(c, fi);
    c.phi[fi] = rhoa * ms;
    c.phiU[fi] = rhoaU * ms + p12 * SfOf(c, fi);
    c.phiE[fi] = rhoah * ms + p12 * umOf(c, fi) * ms;
  }
}

void calcFluxHLLC(Case& c) {
  const int NF = c.F + c.B;
  std::vector<double> rho_l, rho_r, p_l, p_r, c_l, c_r, E_l, E_r, H_l, H_r;
  VolS P = fieldP(c), RHO = fieldRho(c);
  reconstruct(c, RHO, +1, c.cfg.recon_rho, rho_l);
  reconstruct(c, RHO, -1, c.cfg.recon_rho, rho_r);
  reconstruct(c, P, +1, c.cfg.recon_rho, p_l);
  reconstruct(c, P, -1, c.cfg.recon_rho, p_r);
  std::vector<V3> U_l, U_r;
  reconstructU(c, +1, U_l);
  reconstructU(c, -1, U_r);
  VolS cs;
  cs.in.resize(c.N);
  cs.bf.resize(c.B);
  for (int i = 0; i < c.N; ++i) cs.in[i] = std::max(std::sqrt(c.gamma / psiOf(c, c.T[i])), VSMALL);
  for (int b = 0; b < c.B; ++b) cs.bf[b] = std::max(std::sqrt(c.gamma / psiOf(c, c.TB[b])), VSMALL);
  setPlagC(c, cs);
  reconstruct(c, cs, +1, c.cfg.recon_T, c_l);
  reconstruct(c, cs, -1, c.cfg.recon_T, c_r);
  VolS E = fieldE(c);
  reconstruct(c, E, +1, c.cfg.recon_T, E_l);
  reconstruct(c, E, -1, c.cfg.recon_T, E_r);
  VolS H = fieldH(c, E);
  reconstruct(c, H, +1, c.cfg.recon_T, H_l);
  reconstruct(c, H, -1, c.cfg.recon_T, H_r);
  const double gInterp = c.gamma;  // linear interpolation of a uniform gamma
  for (int fi = 0; fi < NF; ++fi) {
    const double ms = magSfOf(c, fi);
    const V3 n = SfOf(c, fi) / ms;
    const double coefR = std::sqrt(std::max(VSMALL, rho_r[fi]) / std::max(VSMALL, rho_l[fi]));
    const V3 uAvg = (coefR * U_r[fi] + U_l[fi]) / (coefR + 1.0);
    const double HAvg = (coefR * H_r[fi] + H_l[fi]) / (coefR + 1.0);
    const double cAvg = std::sqrt(std::fabs((gInterp - 1.0) * (HAvg - 0.5 * magSqr(uAvg))));
    const double um = umOf(c, fi);  // hllcFluxScheme.C:157-161
    const double uMag_l = dot(U_l[fi], n) - um;
    const double uMag_r = dot(U_r[fi], n) - um;
    const double uMagAvg = dot(uAvg, n) - um;
    const double Sl = std::min(uMag_l - c_l[fi], uMagAvg - cAvg);
    const double Sr = std::max(uMag_r + c_r[fi], uMagAvg + cAvg);
    const double rl = rho_l[fi], rr = rho_r[fi], pl = p_l[fi], pr = p_r[fi];
    const double Sm = (rr * uMag_r * (Sr - uMag_r) - rl * uMag_l * (Sl - uMag_l) + pl - pr) /
                      (rr * (Sr - uMag_r) - rl * (Sl - uMag_l));
    const double coefSl = pos0(Sl);
    const double coefSr = neg(Sr);
    const double coefSm = pos0(Sm);
    const double coefSlm = (1.0 - coefSl) * coefSm;
    const double coefSmr = (1.0 - coefSm) * (1.0 - coefSr);
    const double fluxRhoStar_l = Sm / (Sl - Sm) * ((Sl - uMag_l) * rl);
    const double fluxRhoStar_r = Sm / (Sr - Sm) * ((Sr - uMag_r) * rr);
    c.phi[fi] = (coefSl * rl * uMag_l + coefSlm * fluxRhoStar_l + coefSmr * fluxRhoStar_r + coefSr * rr * uMag_r) * ms;
    const double pStar_l = rl * (uMag_l - Sl) * (uMag_l - Sm) + pl;
    const double pStar_r = rr * (uMag_r - Sr) * (uMag_r - Sm) + pr;
    const V3 rhoUStar_l = 1.0 / (Sl - Sm) * ((Sl - uMag_l) * rl * U_l[fi] + (pStar_l - pl) * n);
    const V3 rhoUStar_r = 1.0 / (Sr - Sm) * ((Sr - uMag_r) * rr * U_r[fi] + (pStar_r - pr) * n);
    const V3 fluxRhoUStar_l = Sm * rhoUStar_l + pStar_l * n;
    const V3 fluxRhoUStar_r = Sm * rhoUStar_r + pStar_r * n;
    c.phiU[fi] = (coefSl * (rl * uMag_l * U_l[fi] + pl * n) + coefSlm * fluxRhoUStar_l + coefSmr * fluxRhoUStar_r +
                  coefSr * (rr * uMag_r * U_r[fi] + pr * n)) *
                 ms;
    const double rhoEStar_l = 1.0 / (Sl - Sm) * ((Sl - uMag_l) * (rl * E_l[fi]) - pl * uMag_l + pStar_l * Sm);
    const double rhoEStar_r = 1.0 / (Sr - Sm) * ((Sr - uMag_r) * (rr * E_r[fi]) - pr * uMag_r + pStar_r * Sm);
    const double fluxRhoEStar_l = Sm * (rhoEStar_l + pStar_l) + pStar_l * um;
    const double fluxRhoEStar_r = Sm * (rhoEStar_r + pStar_r) + pStar_r * um;
    c.phiE[fi] = (coefSl * rl * H_l[fi] * uMag_l + coefSlm * fluxRhoEStar_l + coefSmr * fluxRhoEStar_r +
                  coefSr * rr * H_r[fi] * uMag_r) *
                 ms;
  }
}

void calcFluxRoe(Case& c) {
  const int NF = c.F + c.B;
  std::vector<double> rho_l, rho_r, p_l, p_r, E_l, E_r, H_l, H_r;
  VolS P = fieldP(c), RHO = fieldRho(c);
  reconstruct(c, RHO, +1, c.cfg.recon_rho, rho_l);
  reconstruct(c, RHO, -1, c.cfg.recon_rho, rho_r);
  reconstruct(c, P, +1, c.cfg.recon_rho, p_l);
  reconstruct(c, P, -1, c.cfg.recon_rho, p_r);
  std::vector<V3> U_l, U_r;
  reconstructU(c, +1, U_l);
  reconstructU(c, -1, U_r);
  VolS E = fieldE(c);
  reconstruct(c, E, +1, c.cfg.recon_T, E_l);
  reconstruct(c, E, -1, c.cfg.recon_T, E_r);
  VolS H = fieldH(c, E);
  reconstruct(c, H, +1, c.cfg.recon_T, H_l);
  reconstruct(c, H, -1, c.cfg.recon_T, H_r);
  const double gI = c.gamma;
  const double eps = c.cfg.entropy_fix_coeff;
  for (int fi = 0; fi < NF; ++fi) {
    const double ms = magSfOf(c, fi);
    const V3 n = SfOf(c, fi) / ms;
    const double coefR = std::sqrt(std::max(VSMALL, rho_r[fi]) / std::max(VSMALL, rho_l[fi]));
    const double rD = coefR * rho_l[fi];
    const V3 rU = (coefR * U_r[fi] + U_l[fi]) / (coefR + 1.0);
    const double rH = (coefR * H_r[fi] + H_l[fi]) / (coefR + 1.0);
    const double rC = std::sqrt(std::fabs((gI - 1.0) * (rH - 0.5 * magSqr(rU))));
    const double uMag_l = dot(U_l[fi], n), uMag_r = dot(U_r[fi], n);
    const double um = umOf(c, fi);  // roeFluxScheme.C:362-363
    const double uProj = dot(rU, n) - um;
    const V3 rhoU_l = rho_l[fi] * U_l[fi], rhoU_r = rho_r[fi] * U_r[fi];
    const double rhoE_l = rho_l[fi] * E_l[fi], rhoE_r = rho_r[fi] * E_r[fi];
    // getRoeDissipation: P |Lambda| P^-1 assembled in conservative variables
    const double a1 = gI - 1;
    const double theta = 0.5 * a1 * magSqr(rU);
    const double c2 = sqr(rC);
    const double a2 = 1 / (rD * rC * std::sqrt(2.0));
    const double a3 = rD / (rC * std::sqrt(2.0));
    const double a4 = (theta + c2) / a1;
    const double a5 = 1 - theta / c2;
    const double a6 = theta / a1;
    auto cross = [](const V3& a, const V3& b) {
      return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
    };
    // inverse P: rows 1 (vector, 3 rows), 2, 3; columns rho | rhoU | rhoE
    V3 invP11 = (n * a5) - cross(rU, n) / rD;
    T33 invP12 = outer(a1 / c2 * n, rU);
    invP12.a[0][1] += n.z / rD;
    invP12.a[0][2] -= n.y / rD;
    invP12.a[1][0] -= n.z / rD;
    invP12.a[1][2] += n.x / rD;
    invP12.a[2][0] += n.y / rD;
    invP12.a[2][1] -= n.x / rD;
    V3 invP13 = -a1 / c2 * n;
    const double invP21 = a2 * (theta - rC * uProj);
    const V3 invP22 = -a2 * (a1 * rU - rC * n);
    const double invP23 = a1 * a2;
    const double invP31 = a2 * (theta + rC * uProj);
    const V3 invP32 = -a2 * (a1 * rU + rC * n);
    const double invP33 = a1 * a2;
    double L1 = std::fabs(uProj), L2 = std::fabs(uProj + rC), L3 = std::fabs(uProj - rC);
    const double epsilon = eps * std::max(L2, L3);
    if (L1 < epsilon) L1 = (sqr(L1) + sqr(epsilon)) / (2.0 * epsilon);
    if (L2 < epsilon) L2 = (sqr(L2) + sqr(epsilon)) / (2.0 * epsilon);
    if (L3 < epsilon) L3 = (sqr(L3) + sqr(epsilon)) / (2.0 * epsilon);
    const V3 P11 = n;
    const double P12 = a3, P13 = a3;
    T33 P21 = outer(rU, n);
    P21.a[0][1] -= n.z * rD;
    P21.a[0][2] += n.y * rD;
    P21.a[1][0] += n.z * rD;
    P21.a[1][2] -= n.x * rD;
    P21.a[2][0] -= n.y * rD;
    P21.a[2][1] += n.x * rD;
    const V3 P22 = a3 * (rU + rC * n);
    const V3 P23 = a3 * (rU - rC * n);
    const V3 P31 = n * a6 + rD * cross(rU, n);
    const double P32 = a3 * (a4 + rC * uProj);
    const double P33 = a3 * (a4 - rC * uProj);
    // dissipation blocks
    const V3 P11L = P11 * L1;
    const double dCR = dot(P11L, invP11) + (L2 * P12 * invP21) + (L3 * P13 * invP31);
    V3 dCU;  // (P11*L1) & invP12 : vector & tensor = row vector
    for (int j = 0; j < 3; ++j) dCU[j] = P11L.x * invP12.a[0][j] + P11L.y * invP12.a[1][j] + P11L.z * invP12.a[2][j];
    dCU = dCU + (L2 * P12 * invP22) + (L3 * P13 * invP32);
    const double dCE = dot(P11L, invP13) + (L2 * P12 * invP23) + (L3 * P13 * invP33);
    // momentum rows: (P21*L1) & invP11 -> tensor & vector
    T33 P21L;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) P21L.a[i][j] = P21.a[i][j] * L1;
    V3 dMR, dME;
    T33 dMU;
    for (int i = 0; i < 3; ++i) {
      dMR[i] = P21L.a[i][0] * invP11.x + P21L.a[i][1] * invP11.y + P21L.a[i][2] * invP11.z;
      dME[i] = P21L.a[i][0] * invP13.x + P21L.a[i][1] * invP13.y + P21L.a[i][2] * invP13.z;
      for (int j = 0; j < 3; ++j)
        dMU.a[i][j] = P21L.a[i][0] * invP12.a[0][j] + P21L.a[i][1] * invP12.a[1][j] + P21L.a[i][2] * invP12.a[2][j];
    }
    dMR = dMR + (L2 * invP21 * P22) + (L3 * invP31 * P23);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dMU.a[i][j] += (L2 * P22[i] * invP22[j]) + (L3 * P23[i] * invP32[j]);
    dME = dME + (L2 * invP23 * P22) + (L3 * invP33 * P23);
    const V3 P31L = P31 * L1;
    const double dER = dot(P31L, invP11) + (L2 * P32 * invP21) + (L3 * P33 * invP31);
    V3 dEU;
    for (int j = 0; j < 3; ++j) dEU[j] = P31L.x * invP12.a[0][j] + P31L.y * invP12.a[1][j] + P31L.z * invP12.a[2][j];
    dEU = dEU + (L2 * P32 * invP22) + (L3 * P33 * invP32);
    const double dEE = dot(P31L, invP13) + (L2 * P32 * invP23) + (L3 * P33 * invP33);

    const double dRho = rho_r[fi] - rho_l[fi];
    const V3 dRhoU = rhoU_r - rhoU_l;
    const double dRhoE = rhoE_r - rhoE_l;
    double ph = -0.5 * ms * (dCR * dRho + dot(dCU, dRhoU) + dCE * dRhoE);
    V3 tU;
    for (int i = 0; i < 3; ++i)
      tU[i] = dMR[i] * dRho + (dMU.a[i][0] * dRhoU.x + dMU.a[i][1] * dRhoU.y + dMU.a[i][2] * dRhoU.z) + dME[i] * dRhoE;
    V3 pU = -0.5 * ms * tU;
    double pE = -0.5 * ms * (dER * dRho + dot(dEU, dRhoU) + dEE * dRhoE);
    const double rn_l = rho_l[fi] * uMag_l, rn_r = rho_r[fi] * uMag_r;
    ph += 0.5 * ms * (rn_l + rn_r);
    pU = pU + 0.5 * ms * (rn_l * U_l[fi] + rn_r * U_r[fi] + n * (p_l[fi] + p_r[fi]));
    pE += 0.5 * ms * (rn_l * H_l[fi] + rn_r * H_r[fi]);
    if (um != 0.0) {  // roeFluxScheme.C:406-408
      ph -= 0.5 * ms * um * (rho_l[fi] + rho_r[fi]);
      pU = pU - 0.5 * ms * um * (rhoU_l + rhoU_r);
      pE -= 0.5 * ms * um * (rhoE_l + rhoE_r);
    }
    c.phi[fi] = ph;
    c.phiU[fi] = pU;
    c.phiE[fi] = pE;
  }
}

void calcFlux(Case& c) {
  const int NF = c.F + c.B;
  c.phi.assign(NF, 0.0);
  c.phiE.assign(NF, 0.0);
  c.phiU.assign(NF, V3());
  if (c.cfg.flux_scheme == ICS_FLUX_AUSMPLUSUP)
    calcFluxAUSM(c);
  else if (c.cfg.flux_scheme == ICS_FLUX_HLLC)
    calcFluxHLLC(c);
  else
    calcFluxRoe(c);
  for (int b = 0; b < c.B; ++b) c.phiB[b] = c.phi[c.F + b];
}

// ---------------------------------------------------------------------------
// Viscous terms (residualsUpdate.H:16-43): laminar muEff = mu(T) (constant or
// Sutherland As sqrt(T)/(1 + Ts/T)), alphaEff = (Cp/Cv) kappa/Cp with
// kappa = Cp mu / Pr; Gauss linear gradients; Laplacians "Gauss linear
// corrected" (non-orthogonal correction with linearly interpolated
// gradients); boundary snGrad = (psi_b - psi_P) deltaCoeffs_b; boundary
// gradient values corrected to that snGrad (gaussGrad boundary correction).
// ---------------------------------------------------------------------------
struct T9 {
  double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // row-major, a[3*i+j]
};

inline double muOf(const Case& c, double T) {
  if (c.cfg.sutherland) return c.cfg.As * std::sqrt(T) / (1.0 + c.cfg.Ts / T);
  return c.cfg.mu;
}
inline double alphaEffOf(const Case& c, double mu) { return c.cfg.Cp / c.Cv * (mu / c.cfg.Pr); }

// fvc::grad(U) (tensor, (grad U)_ij = d U_j / d x_i) and fvc::grad(e), Gauss linear
void gaussGradVec(const Case& c, const std::vector<V3>& in, const std::vector<V3>& bf, std::vector<T9>& g) {
  g.assign(c.N, T9());
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    for (int j = 0; j < 3; ++j) {
      const double sf = c.w[fi] * (in[o][j] - in[n][j]) + in[n][j];
      for (int i = 0; i < 3; ++i) {
        g[o].a[3 * i + j] += c.Sf[fi][i] * sf;
        g[n].a[3 * i + j] -= c.Sf[fi][i] * sf;
      }
    }
  }
  for (int b = 0; b < c.B; ++b) {
    V3 fb = bf[b];
    if (isCyc(c, b)) {  // coupled: interpolate with the partner's vector rotated (U phase-lagged)
      const V3 up = isPlag(c, b) ? plagVec(c, b, in) : rotP(c, b, in[c.bpartner[b]]);
      const V3& uo = in[c.bcell[b]];
      for (int j = 0; j < 3; ++j) fb[j] = c.bw[b] * (uo[j] - up[j]) + up[j];
    }
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) g[c.bcell[b]].a[3 * i + j] += c.bSf[b][i] * fb[j];
  }
  for (int k = 0; k < c.N; ++k)
    for (int q = 0; q < 9; ++q) g[k].a[q] /= c.V[k];
}

// R T R^T of a tensor with the rotation of boundary face b's patch
inline T9 rotT(const Case& c, int b, const T9& t) {
  const double* R = c.patches[c.bpatch[b]].R;
  T9 o;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) s += R[3 * i + k] * t.a[3 * k + l] * R[3 * j + l];
      o.a[3 * i + j] = s;
    }
  return o;
}

struct Viscous {
  std::vector<double> mu, al, e, muB, alB, eB;
  std::vector<T9> gU, tau;  // cell values
  std::vector<V3> ge;
};

inline T9 devTwoT(const T9& g, double mu) {  // mu dev2(T(g))
  T9 t;
  const double tr = g.a[0] + g.a[4] + g.a[8];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t.a[3 * i + j] = mu * (g.a[3 * j + i] - (i == j ? (2.0 / 3.0) * tr : 0.0));
  return t;
}

void viscousFields(const Case& c, Viscous& v) {
  v.mu.resize(c.N);
  v.al.resize(c.N);
  v.e.resize(c.N);
  v.muB.resize(c.B);
  v.alB.resize(c.B);
  v.eB.resize(c.B);
  for (int i = 0; i < c.N; ++i) {
    v.mu[i] = muOf(c, c.T[i]);
    v.al[i] = alphaEffOf(c, v.mu[i]);
    v.e[i] = c.rhoE[i] / c.rho[i] - 0.5 * magSqr(c.U[i]);
  }
  for (int b = 0; b < c.B; ++b) {
    v.muB[b] = muOf(c, c.TB[b]);
    v.alB[b] = alphaEffOf(c, v.muB[b]);
    v.eB[b] = heOf(c, c.TB[b]);
  }
  gaussGradVec(c, c.U, c.UB, v.gU);
  v.tau.resize(c.N);
  for (int i = 0; i < c.N; ++i) v.tau[i] = devTwoT(v.gU[i], v.mu[i]);
  VolS E;
  E.in = v.e;
  E.bf = v.eB;
  gaussGrad(c, E, v.ge);
}

// Viscous face fluxes out of the owner: momentum (laplacian(mu,U) + div(tauMC))
// and energy (div(sigmaDotU . S) + laplacian(alphaEff, e)), each term kept
// separate as in residualsUpdate.H, plus the LF viscous Jacobian coefficient
// sf2 = 0.5 lambda_v |S| deltaCoeffs (viscousFluxScheme.C:234-247) and the
// coefficients of the non-LF laplacians, muG = (mu_f |S|) deltaCoeffs and
// alG = (alphaEff_f |S|) deltaCoeffs (blockFvOperatorsTemplates.C:398-399),
// mu_b and alphaEff_b on physical boundary faces (viscousFluxScheme.C:57-58).
void viscousFluxes(const Case& c, const Viscous& v, std::vector<V3>& lapU, std::vector<V3>& divTau,
                   std::vector<double>& divSig, std::vector<double>& lapE, std::vector<double>& sf2,
                   std::vector<double>& muG, std::vector<double>& alG) {
  const int NF = c.F + c.B;
  muG.assign(NF, 0.0);
  alG.assign(NF, 0.0);
  lapU.assign(NF, V3());
  divTau.assign(NF, V3());
  divSig.assign(NF, 0.0);
  lapE.assign(NF, 0.0);
  sf2.assign(c.F, 0.0);
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    const double wf = c.w[fi];
    auto lin = [&](double a, double b) { return wf * (a - b) + b; };
    const double muf = lin(v.mu[o], v.mu[n]), alf = lin(v.al[o], v.al[n]);
    const double ms = c.magSf[fi];
    const V3 d = c.C[n] - c.C[o];
    const V3 unit = c.Sf[fi] / ms;
    const V3 kcor = unit - d * c.nodc[fi];  // non-orthogonal correction vector
    T9 gUf, tf;
    for (int q = 0; q < 9; ++q) {
      gUf.a[q] = lin(v.gU[o].a[q], v.gU[n].a[q]);
      tf.a[q] = lin(v.tau[o].a[q], v.tau[n].a[q]);
    }
    V3 Uf, snU;
    for (int j = 0; j < 3; ++j) {
      Uf[j] = lin(c.U[o][j], c.U[n][j]);
      const double corr = kcor.x * gUf.a[j] + kcor.y * gUf.a[3 + j] + kcor.z * gUf.a[6 + j];
      snU[j] = c.nodc[fi] * (c.U[n][j] - c.U[o][j]) + corr;
    }
    lapU[fi] = (muf * ms) * snU;
    for (int j = 0; j < 3; ++j)
      divTau[fi][j] = c.Sf[fi].x * tf.a[j] + c.Sf[fi].y * tf.a[3 + j] + c.Sf[fi].z * tf.a[6 + j];
    V3 sig;
    for (int i = 0; i < 3; ++i) {
      double s = 0;
      for (int j = 0; j < 3; ++j) s += (muf * gUf.a[3 * i + j] + tf.a[3 * i + j]) * Uf[j];
      sig[i] = s;
    }
    divSig[fi] = dot(sig, c.Sf[fi]);
    const V3 gef(lin(v.ge[o].x, v.ge[n].x), lin(v.ge[o].y, v.ge[n].y), lin(v.ge[o].z, v.ge[n].z));
    const double snE = c.nodc[fi] * (v.e[n] - v.e[o]) + dot(kcor, gef);
    lapE[fi] = (alf * ms) * snE;
    const double rhof = lin(c.rho[o], c.rho[n]);
    const double lamv = (muf + alf) / rhof;
    sf2[fi] = 0.5 * lamv * ms * c.dc[fi];
    muG[fi] = muf * ms * c.dc[fi];
    alG[fi] = alf * ms * c.dc[fi];
  }
  if (c.hasCyc) sf2.resize(c.F + c.B, 0.0);  // coupled faces keep their own coefficient
  for (int b = 0; b < c.B; ++b) {
    const int o = c.bcell[b];
    const double ms = c.bmagSf[b];
    const V3 n = c.bSf[b] / ms;
    if (isCyc(c, b)) {
      // coupled face: the internal-face formulas with the partner's vectors
      // and tensors rotated into this side's frame (patchNeighbourField)
      const int pc = c.bpartner[b];
      const double wf = c.bw[b];
      auto lin = [&](double a, double bb) { return wf * (a - bb) + bb; };
      const double muf = lin(v.mu[o], v.mu[pc]), alf = lin(v.al[o], v.al[pc]);
      const V3 kcor = n - c.bdelta[b] * c.bnodc[b];
      const T9 gUp = rotT(c, b, v.gU[pc]), tp = rotT(c, b, v.tau[pc]);
      T9 gUf, tf;
      for (int q = 0; q < 9; ++q) {
        gUf.a[q] = lin(v.gU[o].a[q], gUp.a[q]);
        tf.a[q] = lin(v.tau[o].a[q], tp.a[q]);
      }
      const V3 Up = isPlag(c, b) ? plagVec(c, b, c.U) : rotP(c, b, c.U[pc]);
      V3 Uf, snUc;
      for (int j = 0; j < 3; ++j) {
        Uf[j] = lin(c.U[o][j], Up[j]);
        const double corr = kcor.x * gUf.a[j] + kcor.y * gUf.a[3 + j] + kcor.z * gUf.a[6 + j];
        snUc[j] = c.bnodc[b] * (Up[j] - c.U[o][j]) + corr;
      }
      lapU[c.F + b] = (muf * ms) * snUc;
      for (int j = 0; j < 3; ++j)
        divTau[c.F + b][j] = c.bSf[b].x * tf.a[j] + c.bSf[b].y * tf.a[3 + j] + c.bSf[b].z * tf.a[6 + j];
      V3 sig;
      for (int i = 0; i < 3; ++i) {
        double s = 0;
        for (int j = 0; j < 3; ++j) s += (muf * gUf.a[3 * i + j] + tf.a[3 * i + j]) * Uf[j];
        sig[i] = s;
      }
      divSig[c.F + b] = dot(sig, c.bSf[b]);
      const V3 gep = rotP(c, b, v.ge[pc]);
      const V3 gef(lin(v.ge[o].x, gep.x), lin(v.ge[o].y, gep.y), lin(v.ge[o].z, gep.z));
      const double snEc = c.bnodc[b] * (v.e[pc] - v.e[o]) + dot(kcor, gef);
      lapE[c.F + b] = (alf * ms) * snEc;
      const double rhof = lin(c.rho[o], c.rho[pc]);
      sf2[c.F + b] = 0.5 * ((muf + alf) / rhof) * ms * c.bdc[b];
      muG[c.F + b] = muf * ms * c.bdc[b];
      alG[c.F + b] = alf * ms * c.bdc[b];
      continue;
    }
    muG[c.F + b] = v.muB[b];
    alG[c.F + b] = v.alB[b];
    V3 snU;
    for (int j = 0; j < 3; ++j) snU[j] = (c.UB[b][j] - c.U[o][j]) * c.bdc[b];
    const double snE = (v.eB[b] - v.e[o]) * c.bdc[b];
    // boundary gradient: cell gradient with its normal part replaced by snGrad
    T9 gUb = v.gU[o];
    for (int j = 0; j < 3; ++j) {
      const double ng = n.x * v.gU[o].a[j] + n.y * v.gU[o].a[3 + j] + n.z * v.gU[o].a[6 + j];
      for (int i = 0; i < 3; ++i) gUb.a[3 * i + j] += n[i] * (snU[j] - ng);
    }
    const T9 tb = devTwoT(gUb, v.muB[b]);
    lapU[c.F + b] = (v.muB[b] * ms) * snU;
    for (int j = 0; j < 3; ++j)
      divTau[c.F + b][j] = c.bSf[b].x * tb.a[j] + c.bSf[b].y * tb.a[3 + j] + c.bSf[b].z * tb.a[6 + j];
    V3 sig;
    for (int i = 0; i < 3; ++i) {
      double s = 0;
      for (int j = 0; j < 3; ++j) s += (v.muB[b] * gUb.a[3 * i + j] + tb.a[3 * i + j]) * c.UB[b][j];
      sig[i] = s;
    }
    divSig[c.F + b] = dot(sig, c.bSf[b]);
    lapE[c.F + b] = (v.alB[b] * ms) * snE;
  }
}

// ---------------------------------------------------------------------------
// Dual-time ddt (dualTimeDdtScheme.C:111-126 around Euler/backward/steady)
// ---------------------------------------------------------------------------
struct DdtCoeffs {
  double rDeltaT = 0, coefft = 0, coefft0 = 0, coefft00 = 0;
};
DdtCoeffs ddtCoeffs(const Case& c) {
  DdtCoeffs d;
  if (c.cfg.ddt_scheme == ICS_DDT_STEADY) return d;
  d.rDeltaT = 1.0 / c.cfg.delta_t;
  if (c.cfg.ddt_scheme == ICS_DDT_BACKWARD) {
    const double dt = c.cfg.delta_t;
    const double dt0 = c.timeIndex <= 1 ? GREAT : dt;  // no old-old level on the first step
    d.coefft = 1 + dt / (dt + dt0);
    d.coefft00 = dt * dt / (dt0 * (dt + dt0));
    d.coefft0 = d.coefft + d.coefft00;
  }
  return d;
}
// diag and source of fvm::ddt(W) for one cell and one scalar component
inline void ddtMatrix(const Case& c, const DdtCoeffs& d, int i, double W, double W0, double W00, double& diag,
                      double& source) {
  const double Vc = c.V[i];
  if (c.cfg.ddt_scheme == ICS_DDT_STEADY) {
    diag = 0;
    source = 0;
  } else if (c.cfg.ddt_scheme == ICS_DDT_EULER) {
    diag = d.rDeltaT * Vc;
    source = d.rDeltaT * W0 * Vc;
  } else {
    diag = (d.coefft * d.rDeltaT) * Vc;
    source = d.rDeltaT * Vc * (d.coefft0 * W0 - d.coefft00 * W00);
  }
  diag += c.rPseudoDeltaT[i] * Vc;
  source += c.rPseudoDeltaT[i] * W * Vc;
}

// residualsUpdate.H: source = R*V with R = -div(fluxes) - ddt_phys
void residualSource(Case& c) {
  std::vector<double> divR(c.N, 0.0), divE(c.N, 0.0);
  std::vector<V3> divU(c.N);
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    divR[o] += c.phi[fi];
    divR[n] -= c.phi[fi];
    divU[o] = divU[o] + c.phiU[fi];
    divU[n] = divU[n] - c.phiU[fi];
    divE[o] += c.phiE[fi];
    divE[n] -= c.phiE[fi];
  }
  for (int b = 0; b < c.B; ++b) {
    const int o = c.bcell[b];
    divR[o] += c.phi[c.F + b];
    divU[o] = divU[o] + c.phiU[c.F + b];
    divE[o] += c.phiE[c.F + b];
  }
  // viscous divergences, one per fvc term of residualsUpdate.H:24-42
  std::vector<V3> dLapU, dTau;
  std::vector<double> dSig, dLapE;
  if (c.cfg.viscous) {
    Viscous v;
    viscousFields(c, v);
    std::vector<V3> lapU, divTau;
    std::vector<double> divSig, lapE;
    viscousFluxes(c, v, lapU, divTau, divSig, lapE, c.viscSf2, c.viscMuG, c.viscAlG);
    dLapU.assign(c.N, V3());
    dTau.assign(c.N, V3());
    dSig.assign(c.N, 0.0);
    dLapE.assign(c.N, 0.0);
    for (int fi = 0; fi < c.F; ++fi) {
      const int o = c.own[fi], n = c.nei[fi];
      dLapU[o] = dLapU[o] + lapU[fi];
      dLapU[n] = dLapU[n] - lapU[fi];
      dTau[o] = dTau[o] + divTau[fi];
      dTau[n] = dTau[n] - divTau[fi];
      dSig[o] += divSig[fi];
      dSig[n] -= divSig[fi];
      dLapE[o] += lapE[fi];
      dLapE[n] -= lapE[fi];
    }
    for (int b = 0; b < c.B; ++b) {
      const int o = c.bcell[b];
      dLapU[o] = dLapU[o] + lapU[c.F + b];
      dTau[o] = dTau[o] + divTau[c.F + b];
      dSig[o] += divSig[c.F + b];
      dLapE[o] += lapE[c.F + b];
    }
  }
  double l2 = 0;
  c.src.assign(5 * c.N, 0.0);
  const DdtCoeffs d = ddtCoeffs(c);
  const bool steady = c.cfg.ddt_scheme == ICS_DDT_STEADY;
  for (int i = 0; i < c.N; ++i) {
    const double Vc = c.V[i];
    double rR = -(divR[i] / Vc);
    V3 rU = -1.0 * (divU[i] / Vc);
    double rE = -(divE[i] / Vc);
    l2 += sqr((divR[i] / Vc) * Vc);
    if (c.cfg.viscous) {
      rU = rU + dLapU[i] / Vc;
      rU = rU + dTau[i] / Vc;
      rE += dSig[i] / Vc;
      rE += dLapE[i] / Vc;
    }
    if (!steady) {
      double dg, s;
      ddtMatrix(c, d, i, c.rho[i], c.rho0[i], c.rho00[i], dg, s);
      rR -= (dg * c.rho[i] - s) / Vc;
      for (int k = 0; k < 3; ++k) {
        ddtMatrix(c, d, i, c.rhoU[i][k], c.rhoU0[i][k], c.rhoU00[i][k], dg, s);
        rU[k] -= (dg * c.rhoU[i][k] - s) / Vc;
      }
      ddtMatrix(c, d, i, c.rhoE[i], c.rhoE0[i], c.rhoE00[i], dg, s);
      rE -= (dg * c.rhoE[i] - s) / Vc;
    }
    c.src[5 * i + 0] = rR * Vc;
    c.src[5 * i + 1] = rU.x * Vc;
    c.src[5 * i + 2] = rU.y * Vc;
    c.src[5 * i + 3] = rU.z * Vc;
    c.src[5 * i + 4] = rE * Vc;
    if (c.nInst > 1 && hbInZone(c, i)) {
      // Harmonic Balance source -V sum_K D_JK W_K (HBZoneTemplates.C:39-92),
      // added to R*V (HB residualsUpdate.H:72-74); in the HB zone only, and
      // with cylCoords the momentum combined in cylindrical components at
      // each instance's cell centre (HBZone.C:520-652)
      const int J = i / c.Nc, cl = i % c.Nc;
      double hb[5] = {0, 0, 0, 0, 0};
      V3 cyl;
      for (int K = 0; K < c.nInst; ++K) {
        const int j = K * c.Nc + cl;
        const double d = Vc * c.Dhb[J * c.nInst + K];
        hb[0] -= d * c.rho[j];
        hb[4] -= d * c.rhoE[j];
        if (c.hbCyl) {
          V3 rh, th;
          hbFrame(c, j, rh, th);
          cyl = cyl + V3(dot(c.rhoU[j], rh), dot(c.rhoU[j], th), dot(c.rhoU[j], c.hbAxis)) * d;
        } else {
          hb[1] -= d * c.rhoU[j].x;
          hb[2] -= d * c.rhoU[j].y;
          hb[3] -= d * c.rhoU[j].z;
        }
      }
      if (c.hbCyl) {
        V3 rh, th;
        hbFrame(c, i, rh, th);
        const V3 cart = rh * cyl.x + th * cyl.y + c.hbAxis * cyl.z;
        hb[1] -= cart.x;
        hb[2] -= cart.y;
        hb[3] -= cart.z;
      }
      for (int k = 0; k < 5; ++k) c.src[5 * i + k] = c.src[5 * i + k] + hb[k];
    }
    if (c.mrfOn) {
      // addMRFSource: -(omega x rho U) V with rhoU = rho_ * U_ (convectiveFluxScheme.C:123-129)
      const V3 rU = c.rho[i] * c.U[i];
      const V3 o = c.mrfOm[i];
      const V3 cr(o.y * rU.z - o.z * rU.y, o.z * rU.x - o.x * rU.z, o.x * rU.y - o.y * rU.x);
      for (int k = 0; k < 3; ++k) c.src[5 * i + 1 + k] -= cr[k] * Vc;
    }
  }
  c.lastRhoL2 = std::sqrt(l2);
}

// face wave speed lambda = interp(c) + |interp(U) . n| (setCoAndDeltaT.H:52-54)
void waveSpeed(const Case& c, std::vector<double>& lam) {
  VolS cs;
  cs.in.resize(c.N);
  cs.bf.resize(c.B);
  for (int i = 0; i < c.N; ++i) cs.in[i] = std::sqrt(c.gamma / psiOf(c, c.T[i]));
  for (int b = 0; b < c.B; ++b) cs.bf[b] = std::sqrt(c.gamma / psiOf(c, c.TB[b]));
  setPlagC(c, cs);
  std::vector<double> ci;
  interpLinear(c, cs, ci);
  std::vector<double> ui[3];
  for (int k = 0; k < 3; ++k) interpLinear(c, Ucmpt(c, k), ui[k]);
  lam.resize(c.F + c.B);
  for (int fi = 0; fi < c.F + c.B; ++fi) {
    const V3 n = SfOf(c, fi) / magSfOf(c, fi);
    V3 uf(ui[0][fi], ui[1][fi], ui[2][fi]);
    const int b = fi - c.F;
    if (b >= 0 && isCyc(c, b)) {  // fvc::interpolate(U) on a coupled patch: the partner's U rotated
      const V3 up = isPlag(c, b) ? plagVec(c, b, c.U) : rotP(c, b, c.U[c.bpartner[b]]);
      const V3 uo = c.U[c.bcell[b]];
      const double w = c.bw[b];
      uf = V3(w * (uo.x - up.x) + up.x, w * (uo.y - up.y) + up.y, w * (uo.z - up.z) + up.z);
    }
    lam[fi] = ci[fi] + std::fabs(dot(uf, n) - umOf(c, fi));
  }
}

// sqrt(sum over instances of |s0|^2 + |s1|^2 + |v0|^2), scalars rho, rhoE and
// vector rhoU (setCoAndDeltaT.H:10-16; HB outerLoop.H:34-56)
double residualNorm(const std::vector<double>& r) {
  double s = 0;
  for (size_t J = 0; J < r.size() / 5; ++J) {
    const double* q = &r[5 * J];
    s += sqr(q[0]) + sqr(q[4]) + (sqr(q[1]) + sqr(q[2]) + sqr(q[3]));
  }
  return std::sqrt(s);
}

// setCoAndDeltaT.H
void setCoAndDeltaT(Case& c) {
  if (c.initResValid) {
    const bool firstIter = c.ctl[0].corr == 1;
    if (!firstIter && c.prevResValid) {
      const double normInit = residualNorm(c.initRes);
      const double normPrev = residualNorm(c.prevRes);
      double ratio = normPrev / normInit;
      ratio = std::max(std::min(ratio, c.cfg.pseudo_co_max_increase), c.cfg.pseudo_co_min_decrease);
      for (int i = 0; i < c.N; ++i) {
        c.pseudoCo[i] *= ratio;
        c.pseudoCo[i] = std::max(std::min(c.pseudoCo[i], c.cfg.pseudo_co_num_max), c.cfg.pseudo_co_num_min);
      }
    }
    c.prevRes = c.initRes;
    c.prevResValid = true;
  }
  std::vector<double> lam;
  waveSpeed(c, lam);
  std::fill(c.rPseudoDeltaT.begin(), c.rPseudoDeltaT.end(), 0.0);
  for (int fi = 0; fi < c.F; ++fi) {
    const double frdt = c.nodc[fi] * lam[fi];
    c.rPseudoDeltaT[c.own[fi]] = std::max(c.rPseudoDeltaT[c.own[fi]], frdt);
    c.rPseudoDeltaT[c.nei[fi]] = std::max(c.rPseudoDeltaT[c.nei[fi]], frdt);
  }
  for (int b = 0; b < c.B; ++b) {
    const Patch& pt = c.patches[c.bpatch[b]];
    if (isCyc(c, b)) {  // coupled: nonOrthDeltaCoeffs lambda (setCoAndDeltaT.H:73-87)
      const int o = c.bcell[b];
      c.rPseudoDeltaT[o] = std::max(c.rPseudoDeltaT[o], c.bnodc[b] * lam[c.F + b]);
      continue;
    }
    if (!pt.is_wall) continue;
    const int o = c.bcell[b];
    const double cc = std::sqrt(c.gamma / psiOf(c, c.T[o]));
    const double pl = 0.5 * c.bdc[b] * (cc + std::fabs(dot(c.U[o], c.bSf[b] / c.bmagSf[b]) - umOf(c, c.F + b)));
    c.rPseudoDeltaT[o] = std::max(c.rPseudoDeltaT[o], pl);
  }
  for (int i = 0; i < c.N; ++i) c.rPseudoDeltaT[i] /= c.pseudoCo[i];
  // ddtCoeff = max diag(fvm::ddt(rho|rhoU|rhoE)) / V
  const DdtCoeffs d = ddtCoeffs(c);
  for (int i = 0; i < c.N; ++i) {
    double dg, s;
    ddtMatrix(c, d, i, 0, 0, 0, dg, s);
    c.ddtCoeff[i] = dg / c.V[i];
  }
}

// ---------------------------------------------------------------------------
// Jacobian (convectiveFluxScheme::createConvectiveJacobian)
// ---------------------------------------------------------------------------
// Euler flux Jacobian at state (U, E) for unit normal n (addFluxTerms:432-464)
B5 eulerJacobian(double g, const V3& U, double E, const V3& n) {
  B5 A;
  const double theta = 0.5 * (g - 1) * magSqr(U);
  const double a1 = g * E - theta;
  const double a2 = g - 1;
  const double projU = dot(U, n);
  // d(cont)/d(rhoU) = n
  A(0, 1) = n.x;
  A(0, 2) = n.y;
  A(0, 3) = n.z;
  // d(mom)/d(rho) = n theta - U projU
  for (int i = 0; i < 3; ++i) A(1 + i, 0) = n[i] * theta - U[i] * projU;
  // d(mom)/d(rhoU) = U n - a2 n U + projU I
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A(1 + i, 1 + j) = U[i] * n[j] - a2 * n[i] * U[j] + (i == j ? projU : 0.0);
  // d(mom)/d(rhoE) = n a2
  for (int i = 0; i < 3; ++i) A(1 + i, 4) = n[i] * a2;
  A(4, 0) = projU * (theta - a1);
  for (int j = 0; j < 3; ++j) A(4, 1 + j) = n[j] * a1 - a2 * U[j] * projU;
  A(4, 4) = g * projU;
  return A;
}

const int diagIdx[5] = {0, 6, 12, 18, 24};

void assembleJacobian(Case& c) {
  const int NF = c.F + c.B;
  c.diag.assign(c.N, B5());
  c.lower.assign(c.F, B5());
  c.upper.assign(c.F, B5());
  std::vector<V3> U_l, U_r;
  reconstructU(c, +1, U_l);
  reconstructU(c, -1, U_r);
  VolS E = fieldE(c);
  std::vector<double> E_l, E_r;
  reconstruct(c, E, +1, c.cfg.recon_T, E_l);
  reconstruct(c, E, -1, c.cfg.recon_T, E_r);
  const double g = c.gamma;
  // insertBlock: upper = 0.5|S| A_R, lower = -0.5|S| A_L, negSumDiag
  for (int fi = 0; fi < c.F; ++fi) {
    const V3 n = c.Sf[fi] / c.magSf[fi];
    const B5 AL = eulerJacobian(g, U_l[fi], E_l[fi], n);
    const B5 AR = eulerJacobian(g, U_r[fi], E_r[fi], n);
    const double hs = 0.5 * c.magSf[fi];
    for (int k = 0; k < 25; ++k) {
      const double up = hs * AR.a[k];
      const double lo = -0.5 * c.magSf[fi] * AL.a[k];
      c.upper[fi].a[k] += up;
      c.lower[fi].a[k] += lo;
      c.diag[c.own[fi]].a[k] -= lo;
      c.diag[c.nei[fi]].a[k] -= up;
    }
  }
  // MRF: -div(w, u_MRF |S|) on rho, rhoU (x I), rhoE (convectiveFluxScheme.C:477-481;
  // fvj::div of a face flux, blockFvOperatorsTemplates.C:148-197)
  if (c.mrfOn) {
    for (int fi = 0; fi < c.F; ++fi) {
      const double phm = c.mrfU[fi] * c.magSf[fi];
      const double up = phm * (1 - c.w[fi]), lo = -phm * c.w[fi];
      for (int q = 0; q < 5; ++q) {
        const int k = diagIdx[q];
        c.upper[fi].a[k] -= up;
        c.lower[fi].a[k] -= lo;
        c.diag[c.own[fi]].a[k] -= -lo;
        c.diag[c.nei[fi]].a[k] -= -up;
      }
    }
  }
  // coupled (cyclic) faces: insertBlock's interface block 0.5|S| A_R with
  // diag += 0.5|S| A_L; -div(w, u_MRF |S|): interface -= phi (1-w), diag -= phi w
  // (blockFvMatrix.C:241-262, blockFvOperatorsTemplates.C:176-195)
  if (c.hasCyc) {
    c.iface.assign(c.B, B5());
    for (int b = 0; b < c.B; ++b) {
      if (!isCyc(c, b)) continue;
      const int fi = c.F + b, o = c.bcell[b];
      const V3 n = c.bSf[b] / c.bmagSf[b];
      const B5 AL = eulerJacobian(g, U_l[fi], E_l[fi], n);
      const B5 AR = eulerJacobian(g, U_r[fi], E_r[fi], n);
      for (int k = 0; k < 25; ++k) {
        const double up = 0.5 * c.bmagSf[b] * AR.a[k];
        const double lo = -0.5 * c.bmagSf[b] * AL.a[k];
        c.iface[b].a[k] += up;
        c.diag[o].a[k] -= lo;
      }
      if (c.mrfOn) {
        const double phm = c.mrfU[fi] * c.bmagSf[b];
        const double up = phm * (1 - c.bw[b]), lo = -phm * c.bw[b];
        for (int q = 0; q < 5; ++q) {
          c.iface[b].a[diagIdx[q]] -= up;
          c.diag[o].a[diagIdx[q]] -= -lo;
        }
      }
    }
  }
  // addDissipationJacobian: lambda = interp(c) + |interp(U).n - u_MRF|, subtracted
  std::vector<double> lam;
  waveSpeed(c, lam);
  for (int fi = 0; fi < c.F; ++fi) {
    const double d = 0.5 * c.magSf[fi] * lam[fi];
    for (int q = 0; q < 5; ++q) {
      const int k = diagIdx[q];
      c.upper[fi].a[k] -= d;
      c.lower[fi].a[k] -= d;
      c.diag[c.own[fi]].a[k] += d;
      c.diag[c.nei[fi]].a[k] += d;
    }
  }
  for (int b = 0; b < c.B; ++b) {
    const double d = 0.5 * c.bmagSf[b] * lam[c.F + b];
    for (int q = 0; q < 5; ++q) c.diag[c.bcell[b]].a[diagIdx[q]] += d;
    if (isCyc(c, b))
      for (int q = 0; q < 5; ++q) c.iface[b].a[diagIdx[q]] -= d;
  }
  // addBoundaryTerms (boundaryJacobian :47-120, :219-355)
  for (int b = 0; b < c.B; ++b) {
    const Patch& pt = c.patches[c.bpatch[b]];
    const int ci = c.bcell[b];
    if (isCyc(c, b)) continue;  // physical patches only
    // valueInternalCoeffs
    double pV = 1, tV = 1;
    V3 uV(1, 1, 1);
    const V3 nf = c.bSf[b] / c.bmagSf[b];
    switch (pt.kind) {
      case ICS_PATCH_ZERO_GRADIENT: break;
      case ICS_PATCH_SLIP: uV = V3(1 - std::fabs(nf.x), 1 - std::fabs(nf.y), 1 - std::fabs(nf.z)); break;
      case ICS_PATCH_FIXED: pV = 0; tV = 0; uV = V3(0, 0, 0); break;
      case ICS_PATCH_PRESSURE_OUTLET: pV = 0; break;
      case ICS_PATCH_TOTAL_INLET:
        pV = 0;
        tV = 0;
        if (c.phiB[b] < 0) uV = V3(nf.x * nf.x, nf.y * nf.y, nf.z * nf.z);
        break;
      case ICS_PATCH_ISOTHERMAL_WALL: tV = 0; uV = V3(0, 0, 0); break;
    }
    const V3 SfB = c.bSf[b];
    const double rhoB = rhoBof(c, b);
    const V3 UB = c.UB[b];
    const double UrelBdotSf = dot(UB, SfB) - umOf(c, c.F + b) * c.bmagSf[b];
    const double pB = c.pB[b], TB = c.TB[b];
    const double rhoEB = rhoB * (heOf(c, TB) + 0.5 * magSqr(UB));
    const double cvB = c.Cv;
    const V3 SuV(SfB.x * uV.x, SfB.y * uV.y, SfB.z * uV.z);
    const double dCdp = rhoB / pB * UrelBdotSf * pV;
    const V3 dCdU = rhoB * SuV;
    const double dCdT = -rhoB / TB * UrelBdotSf * tV;
    const V3 dMdp = (rhoB / pB * UB * UrelBdotSf + SfB) * pV;
    T33 dMdU = outer(rhoB * UB, SuV);
    const V3 dMdUDiag = rhoB * UrelBdotSf * uV;
    const V3 dMdT = -rhoB / TB * UB * UrelBdotSf * tV;
    const double dEdp = (rhoEB / pB * UrelBdotSf + dot(UB, SfB)) * pV;
    const V3 dEdU = SuV * (rhoEB + pB) + rhoB * UrelBdotSf * V3(UB.x * uV.x, UB.y * uV.y, UB.z * uV.z);
    const double dEdT = UrelBdotSf * (rhoB * cvB - rhoEB / TB) * tV;
    for (int i = 0; i < 3; ++i) dMdU.a[i][i] += dMdUDiag[i];
    // derivatives of primitives w.r.t. conservative variables of the interior cell
    const double rhoI = c.rho[ci];
    const V3 UI = c.U[ci];
    const double rhoEI = c.rhoE[ci];
    const double gI = c.gamma, cvI = c.Cv;
    const double dPdRho = 0.5 * (gI - 1) * magSqr(UI);
    const V3 dUdRho = -1.0 * UI / rhoI;
    const double dTdRho = -1.0 / (cvI * rhoI) * (rhoEI / rhoI - magSqr(UI));
    const V3 dPdRhoU = -(gI - 1) * UI;
    const double dUdRhoU = 1.0 / rhoI;  // spherical tensor
    const V3 dTdRhoU = -1.0 * UI / (cvI * rhoI);
    const double dPdRhoE = gI - 1;
    const double dTdRhoE = 1.0 / (cvI * rhoI);
    B5& D = c.diag[ci];
    // continuity row
    D(0, 0) += dCdp * dPdRho;
    D(0, 0) += dot(dCdU, dUdRho);
    D(0, 0) += dCdT * dTdRho;
    for (int j = 0; j < 3; ++j) {
      D(0, 1 + j) += dCdp * dPdRhoU[j];
      D(0, 1 + j) += dCdU[j] * dUdRhoU;
      D(0, 1 + j) += dCdT * dTdRhoU[j];
    }
    D(0, 4) += dCdp * dPdRhoE;
    D(0, 4) += 0.0;
    D(0, 4) += dCdT * dTdRhoE;
    // momentum rows
    for (int i = 0; i < 3; ++i) {
      D(1 + i, 0) += dMdp[i] * dPdRho;
      D(1 + i, 0) += dMdU.a[i][0] * dUdRho.x + dMdU.a[i][1] * dUdRho.y + dMdU.a[i][2] * dUdRho.z;
      D(1 + i, 0) += dMdT[i] * dTdRho;
      for (int j = 0; j < 3; ++j) {
        D(1 + i, 1 + j) += dMdp[i] * dPdRhoU[j];
        D(1 + i, 1 + j) += dMdU.a[i][j] * dUdRhoU;
        D(1 + i, 1 + j) += dMdT[i] * dTdRhoU[j];
      }
      D(1 + i, 4) += dMdp[i] * dPdRhoE;
      D(1 + i, 4) += 0.0;
      D(1 + i, 4) += dMdT[i] * dTdRhoE;
    }
    // energy row
    D(4, 0) += dEdp * dPdRho;
    D(4, 0) += dot(dEdU, dUdRho);
    D(4, 0) += dEdT * dTdRho;
    for (int j = 0; j < 3; ++j) {
      D(4, 1 + j) += dEdp * dPdRhoU[j];
      D(4, 1 + j) += dEdU[j] * dUdRhoU;
      D(4, 1 + j) += dEdT * dTdRhoU[j];
    }
    D(4, 4) += dEdp * dPdRhoE;
    D(4, 4) += 0.0;
    D(4, 4) += dEdT * dTdRhoE;
  }
  // addTemporalTerms
  for (int i = 0; i < c.N; ++i) {
    const double dc = c.ddtCoeff[i] * c.V[i];
    for (int q = 0; q < 5; ++q) c.diag[i].a[diagIdx[q]] += dc;
  }
  // addMRFSource: skew(omega) V on the momentum block (convectiveFluxScheme.C:131-137)
  if (c.mrfOn) {
    for (int i = 0; i < c.N; ++i) {
      const V3 o = c.mrfOm[i];
      const double Vc = c.V[i];
      B5& D = c.diag[i];
      D(1, 2) -= o.z * Vc;
      D(1, 3) += o.y * Vc;
      D(2, 1) += o.z * Vc;
      D(2, 3) -= o.x * Vc;
      D(3, 1) -= o.y * Vc;
      D(3, 2) += o.x * Vc;
    }
  }
  // viscousFluxScheme::createViscousJacobian without LaxFriedrichJacobian
  // (viscousFluxScheme.C:249-273): minus the laplacians of mu and alphaEff
  // acting through -U/rho, 1/rho (x I), -E/rho + |U|^2/rho, -U/rho, 1/rho, with
  // E = he(T) + 0.5 |U|^2.  A laplacian of coefficient s and field vf gives
  // upper = vf[nei] s, lower = vf[own] s, diag -= the lower of its own faces
  // (blockFvOperatorsTemplates.C:386-448): so each face adds vf[cell] s to the
  // diagonal of each of its cells and -vf[other] s to the off-diagonal
  // block; a coupled face the interface -vf_b s with vf_b the patch value
  // and vf[cell] s on the diagonal.  Physical patches add the boundary
  // terms of addBoundaryTerms (viscousFluxScheme.C:41-86, 120-215).
  if (c.cfg.viscous && !c.cfg.viscous_lf_jacobian && (int)c.viscMuG.size() == c.F + c.B) {
    // the five laplacian fields at a cell (or patch) state: -U/rho, 1/rho, -E/rho + |U|^2/rho
    struct VF {
      V3 mUr;
      double ir, eR;
    };
    auto vfOf = [&](double rho, const V3& U, double T) {
      VF r;
      const double E = heOf(c, T) + 0.5 * magSqr(U);
      r.mUr = V3(-U.x / rho, -U.y / rho, -U.z / rho);
      r.ir = 1.0 / rho;
      r.eR = -E / rho + magSqr(U) / rho;
      return r;
    };
    // add vf s to block A (sign +1) or subtract (-1): the five laplacians' entries
    auto addLap = [&](B5& A, const VF& f, double mg, double ag, double sign) {
      for (int i = 0; i < 3; ++i) {
        A(1 + i, 0) += sign * (f.mUr[i] * mg);
        A(1 + i, 1 + i) += sign * (f.ir * mg);
        A(4, 1 + i) += sign * (f.mUr[i] * ag);
      }
      A(4, 0) += sign * (f.eR * ag);
      A(4, 4) += sign * (f.ir * ag);
    };
    std::vector<VF> cell(c.N);
    for (int i = 0; i < c.N; ++i) cell[i] = vfOf(c.rho[i], c.U[i], c.T[i]);
    for (int fi = 0; fi < c.F; ++fi) {
      const int o = c.own[fi], n = c.nei[fi];
      const double mg = c.viscMuG[fi], ag = c.viscAlG[fi];
      addLap(c.upper[fi], cell[n], mg, ag, -1.0);
      addLap(c.lower[fi], cell[o], mg, ag, -1.0);
      addLap(c.diag[o], cell[o], mg, ag, 1.0);
      addLap(c.diag[n], cell[n], mg, ag, 1.0);
    }
    for (int b = 0; b < c.B; ++b) {
      const int o = c.bcell[b];
      const Patch& pt = c.patches[c.bpatch[b]];
      if (isCyc(c, b)) {
        const double mg = c.viscMuG[c.F + b], ag = c.viscAlG[c.F + b];
        addLap(c.iface[b], vfOf(rhoBof(c, b), c.UB[b], c.TB[b]), mg, ag, -1.0);
        addLap(c.diag[o], cell[o], mg, ag, 1.0);
        continue;
      }
      if (pt.kind == ICS_PATCH_EMPTY) continue;
      // gradientInternalCoeffs of U and T: fixedValue -deltaCoeffs, zeroGradient 0,
      // slip -deltaCoeffs |n_k| (basicSymmetry snGradTransformDiag),
      // pressureInletOutletVelocity -deltaCoeffs sqrt(|1 - n_k^2|) on inflow faces
      // (directionMixed with valueFraction I - n n), 0 on outflow
      const double dcb = c.bdc[b];
      const V3 nf = c.bSf[b] / c.bmagSf[b];
      V3 uG;
      double tG = 0.0;
      switch (pt.kind) {
        case ICS_PATCH_SLIP: uG = V3(-dcb * std::fabs(nf.x), -dcb * std::fabs(nf.y), -dcb * std::fabs(nf.z)); break;
        case ICS_PATCH_FIXED:
        case ICS_PATCH_ISOTHERMAL_WALL:
          uG = V3(-dcb, -dcb, -dcb);
          tG = -dcb;
          break;
        case ICS_PATCH_TOTAL_INLET:
          if (c.phiB[b] < 0)
            uG = V3(-dcb * std::sqrt(std::fabs(1.0 - nf.x * nf.x)), -dcb * std::sqrt(std::fabs(1.0 - nf.y * nf.y)),
                    -dcb * std::sqrt(std::fabs(1.0 - nf.z * nf.z)));
          tG = -dcb;
          break;
        default: break;
      }
      const double muB = c.viscMuG[c.F + b], alB = c.viscAlG[c.F + b];
      const double ms = c.bmagSf[b];
      const V3 dMdU(-muB * uG.x * ms, -muB * uG.y * ms, -muB * uG.z * ms);
      const double dEdT = -alB * c.Cv * tG * ms;
      const double rhoI = c.rho[o];
      const V3 UI = c.U[o];
      const double EI = heOf(c, c.T[o]) + 0.5 * magSqr(UI);
      const double cvI = c.Cv;
      const double dTdRho = -1.0 / (cvI * rhoI) * (EI - magSqr(UI));
      B5& D = c.diag[o];
      for (int i = 0; i < 3; ++i) {
        D(1 + i, 0) += dMdU[i] * (-UI[i] / rhoI);
        D(1 + i, 1 + i) += dMdU[i] * (1.0 / rhoI);
        D(4, 1 + i) += dEdT * (-UI[i] / (cvI * rhoI));
      }
      D(4, 0) += dEdT * dTdRho;
      D(4, 4) += dEdT * (1.0 / (cvI * rhoI));
    }
  }
  // viscousFluxScheme::createViscousJacobian, LaxFriedrichJacobian:
  // minus laplacian(0.5 lambda_v, 1) on rho, rhoU (x I), rhoE (viscousFluxScheme.C:234-247)
  if (c.cfg.viscous && c.cfg.viscous_lf_jacobian && (int)c.viscSf2.size() >= c.F) {
    for (int fi = 0; fi < c.F; ++fi) {
      const double s = c.viscSf2[fi];
      for (int q = 0; q < 5; ++q) {
        const int k = diagIdx[q];
        c.upper[fi].a[k] -= s;
        c.lower[fi].a[k] -= s;
        c.diag[c.own[fi]].a[k] += s;
        c.diag[c.nei[fi]].a[k] += s;
      }
    }
    // coupled faces: the laplacian's interface and diagonal (blockFvOperatorsTemplates.C:428-448)
    if ((int)c.viscSf2.size() == c.F + c.B)
      for (int b = 0; b < c.B; ++b) {
        if (!isCyc(c, b)) continue;
        const double s = c.viscSf2[c.F + b];
        for (int q = 0; q < 5; ++q) {
          c.iface[b].a[diagIdx[q]] -= s;
          c.diag[c.bcell[b]].a[diagIdx[q]] += s;
        }
      }
  }
  // Harmonic Balance diagonal V D_JJ on every equation (HBZone.C:435-518)
  if (c.nInst > 1) {
    for (int i = 0; i < c.N; ++i) {
      if (!hbInZone(c, i)) continue;
      const int J = i / c.Nc;
      const double d = c.V[i] * c.Dhb[J * c.nInst + J];
      for (int q = 0; q < 5; ++q) c.diag[i].a[diagIdx[q]] += d;
    }
  }
  (void)NF;
  c.haveMatrix = true;
}

// ---------------------------------------------------------------------------
// Linear algebra
// ---------------------------------------------------------------------------
inline void bmv(const B5& A, const double* x, double* y, double sign) {
  for (int i = 0; i < 5; ++i) {
    double s = 0;
    for (int j = 0; j < 5; ++j) s += A(i, j) * x[j];
    y[i] += sign * s;
  }
}

// coupledMatrix::matrixMul -> blockFvMatrix::Amul (face loop in face order)
void matrixMul(const Case& c, const double* x, double* y) {
  for (int i = 0; i < c.N; ++i) {
    for (int k = 0; k < 5; ++k) y[5 * i + k] = 0;
    bmv(c.diag[i], x + 5 * i, y + 5 * i, 1.0);
  }
  for (int fi = 0; fi < c.F; ++fi) {
    const int l = c.own[fi], u = c.nei[fi];
    bmv(c.lower[fi], x + 5 * l, y + 5 * u, 1.0);
    bmv(c.upper[fi], x + 5 * u, y + 5 * l, 1.0);
  }
  // Harmonic Balance coupling blocks (J, K != J): V D_JK times the identity
  // on every equation (dbnsFullyImplicitHBFoam outerLoop.H, HB.addBlock)
  if (c.nInst > 1) {
    for (int i = 0; i < c.N; ++i) {
      if (!hbInZone(c, i)) continue;
      const int J = i / c.Nc, cl = i % c.Nc;
      for (int K = 0; K < c.nInst; ++K) {
        if (K == J) continue;
        const double d = c.V[i] * c.Dhb[J * c.nInst + K];
        const double* xk = x + 5 * (K * c.Nc + cl);
        for (int k = 0; k < 5; ++k) y[5 * i + k] += d * xk[k];
      }
    }
  }
  // cyclic interfaces (blockFvMatrix::Amul, blockFvMatrix.C:386-407): the
  // partner's unknowns with the momentum rotated into this side's frame
  if (c.hasCyc && (int)c.iface.size() == c.B) {
    for (int b = 0; b < c.B; ++b) {
      if (!isCyc(c, b)) continue;
      const int o = c.bcell[b], pc = c.bpartner[b];
      const V3 xu = rotP(c, b, V3(x[5 * pc + 1], x[5 * pc + 2], x[5 * pc + 3]));
      const double xt[5] = {x[5 * pc], xu.x, xu.y, xu.z, x[5 * pc + 4]};
      bmv(c.iface[b], xt, y + 5 * o, 1.0);
    }
  }
}

// lusgs.C:50-127 scalar diagonal
bool lusgsDiag(const Case& c, std::vector<double>& rD) {
  // scalars (rho, rhoE) first, then the vector diagonal xx, yy, zz
  const int order[5] = {0, 24, 6, 12, 18};
  rD.assign(c.N, GREAT);
  for (int i = 0; i < c.N; ++i) {
    for (int q = 0; q < 5; ++q) rD[i] = 1.0 / std::max(1.0 / rD[i], std::fabs(c.diag[i].a[order[q]]));
    if (rD[i] < VSMALL) return false;
  }
  return true;
}

// lusgs::precondition (lusgs.C:220-385), sequential in cell order
void lusgsPrecondition(const Case& c, const std::vector<double>& rD, double* r) {
  for (int ci = 0; ci < c.N; ++ci) {
    double d[5];
    for (int k = 0; k < 5; ++k) d[k] = rD[ci] * r[5 * ci + k];
    for (int fi : c.cellFaces[ci]) {
      if (c.own[fi] == ci && c.nei[fi] > ci) bmv(c.lower[fi], d, r + 5 * c.nei[fi], -1.0);
    }
  }
  for (int ci = c.N - 1; ci >= 0; --ci) {
    double d[5];
    for (int k = 0; k < 5; ++k) d[k] = rD[ci] * r[5 * ci + k];
    for (int k = 0; k < 5; ++k) r[5 * ci + k] = d[k];
    for (int fi : c.cellFaces[ci]) {
      if (c.nei[fi] == ci && c.own[fi] < ci) bmv(c.upper[fi], d, r + 5 * c.own[fi], -1.0);
    }
  }
}

// 5x5 inverse by LU with partial pivoting (LUscalarMatrix restated)
bool inv5(const B5& A, B5& Ainv) {
  double a[5][5];
  int piv[5];
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) a[i][j] = A(i, j);
  for (int k = 0; k < 5; ++k) {
    int p = k;
    double m = std::fabs(a[k][k]);
    for (int i = k + 1; i < 5; ++i)
      if (std::fabs(a[i][k]) > m) {
        m = std::fabs(a[i][k]);
        p = i;
      }
    piv[k] = p;
    if (m == 0) return false;
    if (p != k)
      for (int j = 0; j < 5; ++j) std::swap(a[k][j], a[p][j]);
    for (int i = k + 1; i < 5; ++i) {
      a[i][k] /= a[k][k];
      for (int j = k + 1; j < 5; ++j) a[i][j] -= a[i][k] * a[k][j];
    }
  }
  for (int col = 0; col < 5; ++col) {
    double b[5] = {0, 0, 0, 0, 0};
    b[col] = 1;
    for (int k = 0; k < 5; ++k)
      if (piv[k] != k) std::swap(b[k], b[piv[k]]);
    for (int i = 1; i < 5; ++i)
      for (int j = 0; j < i; ++j) b[i] -= a[i][j] * b[j];
    for (int i = 4; i >= 0; --i) {
      for (int j = i + 1; j < 5; ++j) b[i] -= a[i][j] * b[j];
      b[i] /= a[i][i];
    }
    for (int i = 0; i < 5; ++i) Ainv(i, col) = b[i];
  }
  return true;
}

void jacobiPrecondition(const Case& c, double* r) {
  for (int i = 0; i < c.N; ++i) {
    B5 inv;
    inv5(c.diag[i], inv);
    double z[5] = {0, 0, 0, 0, 0};
    bmv(inv, r + 5 * i, z, 1.0);
    for (int k = 0; k < 5; ++k) r[5 * i + k] = z[k];
  }
}

int precondition(const Case& c, const std::vector<double>& rD, double* r) {
  if (c.cfg.preconditioner == ICS_PC_LUSGS)
    lusgsPrecondition(c, rD, r);
  else if (c.cfg.preconditioner == ICS_PC_JACOBI)
    jacobiPrecondition(c, r);
  return ICS_OK;
}

// residualsIO helpers: per-equation L1 with scalar (rho, rhoE) and vector (rhoU) norm factors
// residualsIO of the coupled system: one entry per equation and instance,
// [5*J + k] (the reference's 2 nO scalars and nO vectors)
struct ResIO {
  std::vector<double> init, fin;
  int nIter = 0;
};

// L1 residuals per instance: scalars rho, rhoE normalised by their own
// factor, the three rhoU components by the vector factor (residualsIO.H)
void l1ResidualIO(const Case& c, const double* r, const std::vector<double>& nf, std::vector<double>& out) {
  out.assign(5 * c.nInst, 0.0);
  for (int J = 0; J < c.nInst; ++J) {
    double s0 = 0, s1 = 0, vx = 0, vy = 0, vz = 0;
    for (int i = J * c.Nc; i < (J + 1) * c.Nc; ++i) {
      s0 += std::fabs(r[5 * i + 0]);
      vx += std::fabs(r[5 * i + 1]);
      vy += std::fabs(r[5 * i + 2]);
      vz += std::fabs(r[5 * i + 3]);
      s1 += std::fabs(r[5 * i + 4]);
    }
    double* o = &out[5 * J];
    o[0] = s0 / nf[3 * J];
    o[4] = s1 / nf[3 * J + 1];
    o[1] = vx / nf[3 * J + 2];
    o[2] = vy / nf[3 * J + 2];
    o[3] = vz / nf[3 * J + 2];
  }
}

// norm factors sum |A (W - avg W)| + |b| per instance (gmres.C:812-850;
// gAverage per field, i.e. per instance) and the initial residuals
void normFactorsIO(const Case& c, const std::vector<double>& W, std::vector<double>& nf, ResIO& res) {
  const int n5 = 5 * c.N;
  const double* b = c.src.data();
  std::vector<double> wmr(n5), tmp(n5);
  for (int J = 0; J < c.nInst; ++J) {
    double avg[5] = {0, 0, 0, 0, 0};
    for (int i = J * c.Nc; i < (J + 1) * c.Nc; ++i)
      for (int k = 0; k < 5; ++k) avg[k] += W[5 * i + k];
    for (int k = 0; k < 5; ++k) avg[k] /= c.Nc;
    for (int i = J * c.Nc; i < (J + 1) * c.Nc; ++i)
      for (int k = 0; k < 5; ++k) wmr[5 * i + k] = W[5 * i + k] - avg[k];
  }
  matrixMul(c, wmr.data(), tmp.data());
  nf.assign(3 * c.nInst, 0.0);
  for (int J = 0; J < c.nInst; ++J) {
    double* f = &nf[3 * J];
    for (int i = J * c.Nc; i < (J + 1) * c.Nc; ++i) {
      f[0] += std::fabs(tmp[5 * i]) + std::fabs(b[5 * i]);
      f[1] += std::fabs(tmp[5 * i + 4]) + std::fabs(b[5 * i + 4]);
      const V3 t(tmp[5 * i + 1], tmp[5 * i + 2], tmp[5 * i + 3]);
      const V3 s(b[5 * i + 1], b[5 * i + 2], b[5 * i + 3]);
      f[2] += mag(t) + mag(s);
    }
    for (int k = 0; k < 3; ++k) f[k] += VSMALL;
  }
  l1ResidualIO(c, b, nf, res.init);
  res.fin = res.init;
  res.nIter = 0;
}

void zeroEmpty(const Case& c, std::vector<double>& r) {
  for (int J = 0; J < c.nInst; ++J)
    for (int k = 0; k < 3; ++k)
      if (c.solD[k] == -1) r[5 * J + 1 + k] = 0.0;
}

// coupledMatrix::solver::stop (coupledMatrixSolver.C:198-221) over all entries
bool stopTest(const Case& c, const ResIO& r) {
  if (r.nIter < c.cfg.min_iter) return false;
  double mx = -VGREAT, mrel = -VGREAT;
  for (double v : r.fin) mx = std::max(mx, v);
  for (int J = 0; J < c.nInst; ++J) {
    const double* in = &r.init[5 * J];
    const double* fi = &r.fin[5 * J];
    mrel = std::max(mrel, fi[0] / (in[0] + ROOTVSMALL));
    mrel = std::max(mrel, fi[4] / (in[4] + ROOTVSMALL));
    for (int k = 0; k < 3; ++k)
      if (c.solD[k] == 1) mrel = std::max(mrel, fi[1 + k] / (in[1 + k] + ROOTVSMALL));
  }
  return r.nIter >= c.cfg.max_iter || mx < c.cfg.tolerance || mrel < c.cfg.rel_tol;
}

// the C ABI's 5-entry summary: maximum over instances per equation
void toPerf(const ResIO& r, ics_solver_perf& p) {
  std::memset(&p, 0, sizeof(p));
  for (int k = 0; k < 5; ++k) {
    p.init_res[k] = -VGREAT;
    p.final_res[k] = -VGREAT;
    for (size_t J = 0; J < r.init.size() / 5; ++J) {
      p.init_res[k] = std::max(p.init_res[k], r.init[5 * J + k]);
      p.final_res[k] = std::max(p.final_res[k], r.fin[5 * J + k]);
    }
  }
  p.n_iterations = r.nIter;
}

// gmres::solveDelta (gmres.C:772-1107)
int gmresSolveDelta(Case& c, const std::vector<double>& W, ResIO& perf, std::vector<double>& dx) {
  const int N = c.N, m = c.cfg.n_directions;
  const int n5 = 5 * N;
  const double* b = c.src.data();
  std::vector<double> nf;
  normFactorsIO(c, W, nf, perf);

  std::vector<double> rD;
  if (c.cfg.preconditioner == ICS_PC_LUSGS && !lusgsDiag(c, rD)) {
    c.err = "All diagonals of coupledMatrix are zero";
    return ICS_ERR_DIAG;
  }
  dx.assign(n5, 0.0);
  std::vector<double> r(b, b + n5);
  std::vector<std::vector<double>> Vk(m, std::vector<double>(n5));
  std::vector<double> H(m * m, 0.0), yh(m, 0.0), bh(m + 1, 0.0), cs(m, 0.0), sn(m, 0.0);
  auto givens = [](double h, double beta, double& cc, double& ss) {
    if (beta == 0) {
      cc = 1;
      ss = 0;
    } else if (std::fabs(beta) > std::fabs(h)) {
      double tau = -h / beta;
      ss = 1.0 / std::sqrt(1.0 + sqr(tau));
      cc = ss * tau;
    } else {
      double tau = -beta / h;
      cc = 1.0 / std::sqrt(1.0 + sqr(tau));
      ss = cc * tau;
    }
  };
  int status = ICS_OK;
  do {
    precondition(c, rD, r.data());
    double beta = 0;
    for (int i = 0; i < N; ++i) beta += sqr(r[5 * i]);
    for (int i = 0; i < N; ++i) beta += sqr(r[5 * i + 4]);
    for (int i = 0; i < N; ++i) beta += sqr(r[5 * i + 1]) + sqr(r[5 * i + 2]) + sqr(r[5 * i + 3]);
    beta = std::sqrt(beta);
    if (!(beta > 0) || !std::isfinite(beta)) {
      // the reference divides by beta and produces NaN; stop with a status
      status = std::isfinite(beta) ? ICS_ERR_BREAKDOWN : ICS_ERR_NONFINITE;
      perf.nIter++;
      break;
    }
    std::fill(bh.begin(), bh.end(), 0.0);
    bh[0] = beta;
    for (int i = 0; i < m; ++i) {
      for (int q = 0; q < n5; ++q) Vk[i][q] = r[q] / beta;
      matrixMul(c, Vk[i].data(), r.data());
      precondition(c, rD, r.data());
      for (int j = 0; j <= i; ++j) {
        double s = 0;
        for (int q = 0; q < N; ++q) s += r[5 * q] * Vk[j][5 * q];
        for (int q = 0; q < N; ++q) s += r[5 * q + 4] * Vk[j][5 * q + 4];
        for (int q = 0; q < N; ++q)
          s += r[5 * q + 1] * Vk[j][5 * q + 1] + r[5 * q + 2] * Vk[j][5 * q + 2] + r[5 * q + 3] * Vk[j][5 * q + 3];
        H[j * m + i] = s;
        for (int q = 0; q < n5; ++q) r[q] -= H[j * m + i] * Vk[j][q];
      }
      beta = 0;
      for (int q = 0; q < N; ++q) beta += sqr(r[5 * q]);
      for (int q = 0; q < N; ++q) beta += sqr(r[5 * q + 4]);
      for (int q = 0; q < N; ++q) beta += sqr(r[5 * q + 1]) + sqr(r[5 * q + 2]) + sqr(r[5 * q + 3]);
      beta = std::sqrt(beta);
      for (int j = 0; j < i; ++j) {
        const double Hji = H[j * m + i];
        H[j * m + i] = cs[j] * Hji - sn[j] * H[(j + 1) * m + i];
        H[(j + 1) * m + i] = sn[j] * Hji + cs[j] * H[(j + 1) * m + i];
      }
      givens(H[i * m + i], beta, cs[i], sn[i]);
      const double bhi = bh[i];
      bh[i] = cs[i] * bhi - sn[i] * bh[i + 1];
      bh[i + 1] = sn[i] * bhi + cs[i] * bh[i + 1];
      H[i * m + i] = cs[i] * H[i * m + i] - sn[i] * beta;
    }
    for (int i = m - 1; i >= 0; --i) {
      double sum = bh[i];
      for (int j = i + 1; j < m; ++j) sum -= H[i * m + j] * yh[j];
      double hii = H[i * m + i];
      // stabilise(H_ii, VSMALL)
      double st = hii >= 0 ? hii + VSMALL : hii - VSMALL;
      yh[i] = sum / st;
    }
    for (int i = 0; i < m; ++i)
      for (int q = 0; q < n5; ++q) dx[q] += yh[i] * Vk[i][q];
    matrixMul(c, dx.data(), r.data());
    for (int q = 0; q < n5; ++q) r[q] = b[q] - r[q];
    l1ResidualIO(c, r.data(), nf, perf.fin);
    zeroEmpty(c, perf.fin);
    perf.nIter++;
  } while (!stopTest(c, perf));
  // zero increments in empty directions (coupledMatrix.C:370-381)
  for (int k = 0; k < 3; ++k)
    if (c.solD[k] == -1)
      for (int i = 0; i < N; ++i) dx[5 * i + 1 + k] = 0.0;
  return status;
}

// smoothSolverCoupled::solveDelta (smoothSolverCoupled.C:369-515) with the
// Jacobi smoother (JacobiSmoother.C:42-205): same norm factors as GMRES, then
// nSweeps sweeps x <- D^-1 (b - (A - D) x) between stop tests.
int smoothSolveDelta(Case& c, const std::vector<double>& W, ResIO& perf, std::vector<double>& dx) {
  const int N = c.N, n5 = 5 * N;
  const double* b = c.src.data();
  std::vector<double> nf;
  normFactorsIO(c, W, nf, perf);
  std::vector<double> tmp(n5);
  std::vector<B5> inv(N);
  for (int i = 0; i < N; ++i)
    if (!inv5(c.diag[i], inv[i])) {
      c.err = "singular diagonal block";
      return ICS_ERR_DIAG;
    }
  dx.assign(n5, 0.0);
  std::vector<double> r(n5);
  do {
    for (int s = 0; s < c.cfg.n_sweeps; ++s) {
      // t = (A - D) x  (matrixMulNoDiag), then x = D^-1 (b - t)
      std::fill(tmp.begin(), tmp.end(), 0.0);
      for (int fi = 0; fi < c.F; ++fi) {
        const int l = c.own[fi], u = c.nei[fi];
        bmv(c.lower[fi], dx.data() + 5 * l, tmp.data() + 5 * u, 1.0);
        bmv(c.upper[fi], dx.data() + 5 * u, tmp.data() + 5 * l, 1.0);
      }
      for (int i = 0; i < N; ++i) {
        double t[5];
        for (int k = 0; k < 5; ++k) t[k] = -(tmp[5 * i + k] - b[5 * i + k]);
        double z[5] = {0, 0, 0, 0, 0};
        bmv(inv[i], t, z, 1.0);
        for (int k = 0; k < 5; ++k) dx[5 * i + k] = z[k];
      }
    }
    matrixMul(c, dx.data(), r.data());
    for (int q = 0; q < n5; ++q) r[q] = b[q] - r[q];
    l1ResidualIO(c, r.data(), nf, perf.fin);
    zeroEmpty(c, perf.fin);
    perf.nIter += c.cfg.n_sweeps;
  } while (!stopTest(c, perf));
  for (int k = 0; k < 3; ++k)
    if (c.solD[k] == -1)
      for (int i = 0; i < N; ++i) dx[5 * i + 1 + k] = 0.0;
  return ICS_OK;
}

// ---------------------------------------------------------------------------
// Boundary conditions and field update (updateFields.H)
// ---------------------------------------------------------------------------
void correctBoundaryConditions(Case& c, const std::vector<double>& psiB) {
  const double g = c.gamma;
  // p
  for (int b = 0; b < c.B; ++b) {
    const Patch& pt = c.patches[c.bpatch[b]];
    const int ci = c.bcell[b];
    switch (pt.kind) {
      case ICS_PATCH_ZERO_GRADIENT:
      case ICS_PATCH_SLIP:
      case ICS_PATCH_ISOTHERMAL_WALL: c.pB[b] = c.p[ci]; break;
      case ICS_PATCH_FIXED:
      case ICS_PATCH_PRESSURE_OUTLET: c.pB[b] = pt.p; break;
      case ICS_PATCH_TOTAL_INLET: {
        const double gM1ByG = (g - 1.0) / g;
        c.pB[b] = pt.p0 / std::pow((1.0 + 0.5 * psiB[b] * gM1ByG * (1.0 - pos0(c.phiB[b])) * magSqr(c.UB[b])),
                                   1.0 / gM1ByG);
        break;
      }
      case ICS_PATCH_CYCLIC: {  // coupledFvPatchField::evaluate
        const double pn = isPlag(c, b) ? plagSum(c, b, [&](int q) { return c.p[q]; }) : c.p[c.bpartner[b]];
        c.pB[b] = c.bw[b] * (c.p[ci] - pn) + pn;
        break;
      }
    }
  }
  // U
  for (int b = 0; b < c.B; ++b) {
    const Patch& pt = c.patches[c.bpatch[b]];
    const int ci = c.bcell[b];
    const V3 n = c.bSf[b] / c.bmagSf[b];
    switch (pt.kind) {
      case ICS_PATCH_ZERO_GRADIENT:
      case ICS_PATCH_PRESSURE_OUTLET: c.UB[b] = c.U[ci]; break;
      case ICS_PATCH_SLIP: c.UB[b] = c.U[ci] - n * dot(n, c.U[ci]); break;
      case ICS_PATCH_FIXED: c.UB[b] = V3(pt.U[0], pt.U[1], pt.U[2]); break;
      case ICS_PATCH_ISOTHERMAL_WALL: c.UB[b] = V3(0, 0, 0); break;
      case ICS_PATCH_TOTAL_INLET: {
        // directionMixed with valueFraction = neg(phi)(I - nn), refValue = 0
        const double vf = neg(c.phiB[b]);
        V3 out;
        for (int i = 0; i < 3; ++i) {
          double s = 0;
          for (int j = 0; j < 3; ++j) {
            const double Iij = (i == j ? 1.0 : 0.0);
            const double vfij = vf * (Iij - n[i] * n[j]);
            s += (Iij - vfij) * c.U[ci][j];
          }
          out[i] = 0.0 + s;
        }
        c.UB[b] = out;
        break;
      }
      case ICS_PATCH_CYCLIC: {  // the partner's velocity rotated into this side's frame
        const V3 up = isPlag(c, b) ? plagVec(c, b, c.U) : rotP(c, b, c.U[c.bpartner[b]]);
        const double w = c.bw[b];
        c.UB[b] = V3(w * (c.U[ci].x - up.x) + up.x, w * (c.U[ci].y - up.y) + up.y, w * (c.U[ci].z - up.z) + up.z);
        break;
      }
    }
  }
  // MRF: a fixedValue patch keeps the frame velocity correctBoundaryVelocity
  // gave it; the HB solver re-assigns every included face here
  // (dbnsFullyImplicitHBFoam updateFields.H:86-88)
  if (c.mrfOn)
    for (int b = 0; b < c.B; ++b) {
      const int kind = c.patches[c.bpatch[b]].kind;
      if (c.mrfBIn[b] && (c.mrfEvery || kind == ICS_PATCH_FIXED || kind == ICS_PATCH_ISOTHERMAL_WALL))
        c.UB[b] = c.mrfBU[b];
    }
  // T
  for (int b = 0; b < c.B; ++b) {
    const Patch& pt = c.patches[c.bpatch[b]];
    const int ci = c.bcell[b];
    switch (pt.kind) {
      case ICS_PATCH_ZERO_GRADIENT:
      case ICS_PATCH_SLIP:
      case ICS_PATCH_PRESSURE_OUTLET: c.TB[b] = c.T[ci]; break;
      case ICS_PATCH_FIXED:
      case ICS_PATCH_ISOTHERMAL_WALL: c.TB[b] = pt.T; break;
      case ICS_PATCH_TOTAL_INLET: {
        const double gM1ByG = (g - 1.0) / g;
        c.TB[b] = pt.T0 / (1.0 + 0.5 * psiB[b] * gM1ByG * (1.0 - pos0(c.phiB[b])) * magSqr(c.UB[b]));
        break;
      }
      case ICS_PATCH_CYCLIC: {
        const int pc = c.bpartner[b];
        c.TB[b] = c.bw[b] * (c.T[ci] - c.T[pc]) + c.T[pc];
        break;
      }
    }
    c.TB[b] = std::max(c.TB[b], c.cfg.T_min);
    if (c.cfg.T_max < GREAT) c.TB[b] = std::max(c.TB[b], c.cfg.T_max);  // updateFields.H:86-89 as written
  }
}

// updateFields.H: W += dW, bounding, thermo, primitives, BCs
int updateFields(Case& c, const std::vector<double>& dW, int& bounded) {
  bounded = 0;
  for (int i = 0; i < c.N; ++i) {
    c.rho[i] += dW[5 * i];
    c.rhoU[i] = c.rhoU[i] + V3(dW[5 * i + 1], dW[5 * i + 2], dW[5 * i + 3]);
    c.rhoE[i] += dW[5 * i + 4];
  }
  bool anyLow = false;
  for (int i = 0; i < c.N; ++i)
    if (c.rho[i] < c.cfg.rho_min) anyLow = true;
  if (anyLow)
    for (int i = 0; i < c.N; ++i) c.rho[i] = std::max(c.rho[i], c.cfg.rho_min);
  const double eMin = heOf(c, c.cfg.T_min);
  const double eMax = heOf(c, c.cfg.T_max);
  for (int i = 0; i < c.N; ++i) {
    c.U[i] = c.rhoU[i] / c.rho[i];
    c.e[i] = c.rhoE[i] / c.rho[i] - 0.5 * magSqr(c.U[i]);
    if (c.e[i] < eMin) {
      c.e[i] = eMin;
      bounded++;
    }
    if (c.cfg.T_max < GREAT && c.e[i] > eMax) {
      c.e[i] = eMax;
      bounded++;
    }
  }
  // thermo.correct(): T from e, psi; boundary psi from the current boundary T
  std::vector<double> psiB(c.B);
  for (int i = 0; i < c.N; ++i) c.T[i] = c.e[i] / c.Cv;
  for (int b = 0; b < c.B; ++b) psiB[b] = psiOf(c, c.TB[b]);
  for (int i = 0; i < c.N; ++i) {
    c.p[i] = c.rho[i] / psiOf(c, c.T[i]);
    c.rhoU[i] = c.rho[i] * c.U[i];
    c.rhoE[i] = c.rho[i] * (c.e[i] + 0.5 * magSqr(c.U[i]));
  }
  correctBoundaryConditions(c, psiB);
  bool finite = true;
  for (int i = 0; i < c.N; ++i)
    if (!std::isfinite(c.rho[i]) || !std::isfinite(c.rhoE[i])) finite = false;
  return finite ? ICS_OK : ICS_ERR_NONFINITE;
}

// boundLocalTimeStep.H (inert unless W_prev produces sub-bound values)
void boundLocalTimeStep(Case& c) {
  if (!c.cfg.local_timestepping || !c.cfg.local_timestepping_bounding) return;
  const double lb = c.cfg.local_timestepping_lower_bound;
  std::vector<double> rhoMin(c.N), eMin(c.N), eT(c.N), factor(c.N, 1.0);
  for (int i = 0; i < c.N; ++i) {
    const double rp = c.Wprev[5 * i], rEp = c.Wprev[5 * i + 4];
    const V3 rUp(c.Wprev[5 * i + 1], c.Wprev[5 * i + 2], c.Wprev[5 * i + 3]);
    rhoMin[i] = lb * rp;
    eMin[i] = lb * (rEp / rp - 0.5 * magSqr(rUp / rp));
    eT[i] = c.rhoE[i] / c.rho[i] - 0.5 * magSqr(c.rhoU[i] / c.rho[i]);
  }
  auto bad = [&](int i) { return c.rho[i] < rhoMin[i] || eT[i] < eMin[i] || eT[i] < SMALL; };
  for (int fi = 0; fi < c.F; ++fi) {
    const int o = c.own[fi], n = c.nei[fi];
    if (bad(o)) {
      factor[o] = std::min(0.5, factor[o]);
      factor[n] = std::min(0.75, factor[n]);
    }
    if (bad(n)) {
      factor[n] = std::min(0.5, factor[n]);
      factor[o] = std::min(0.75, factor[o]);
    }
  }
  for (int i = 0; i < c.N; ++i) c.pseudoCo[i] *= factor[i];
}

void storeW(const Case& c, std::vector<double>& W) {
  W.resize(5 * c.N);
  for (int i = 0; i < c.N; ++i) {
    W[5 * i] = c.rho[i];
    W[5 * i + 1] = c.rhoU[i].x;
    W[5 * i + 2] = c.rhoU[i].y;
    W[5 * i + 3] = c.rhoU[i].z;
    W[5 * i + 4] = c.rhoE[i];
  }
}

// pseudotimeControl::criteriaSatisfied / loop (pseudotimeControl.C), the
// residuals being the initial residuals of the last linear solve
bool criteriaSatisfied(const Case& c, Case::Control& q) {
  const bool finalIter = q.converged || (q.corr == c.cfg.n_pseudo_corr);
  if (q.firstIteration || q.corr == 1 || finalIter) {
    q.firstIteration = false;
    return false;
  }
  const bool storeIni = q.corr == 2;
  if (storeIni) std::memcpy(q.initResiduals, q.residuals, sizeof(q.residuals));
  double mx = -VGREAT, mrel = -VGREAT;
  for (int k = 0; k < 5; ++k) {
    mx = std::max(mx, q.residuals[k]);
    mrel = std::max(mrel, q.residuals[k] / (q.initResiduals[k] + ROOTVSMALL));
  }
  const bool absCheck = mx < c.cfg.pseudo_tol;
  const bool relCheck = !storeIni && mrel < c.cfg.pseudo_tol_rel;
  return (q.corr >= c.cfg.n_pseudo_corr_min) && (absCheck || relCheck);
}
bool pseudoLoopOne(const Case& c, Case::Control& q) {
  const bool steady = c.cfg.ddt_scheme == ICS_DDT_STEADY;
  q.corr++;
  if (!steady && q.corr == c.cfg.n_pseudo_corr + 1) {
    q.corr = 0;
    return false;
  }
  bool completed = false;
  if (q.converged || criteriaSatisfied(c, q)) {
    if (q.converged) {
      q.corr = 0;
      q.converged = false;
      completed = true;
    } else {
      q.converged = true;
    }
  } else {
    completed = false;
  }
  return !completed;
}
// every instance's control is advanced (no short cut); more while any is
bool pseudoLoop(Case& c) {
  bool more = false;
  for (auto& q : c.ctl) more = pseudoLoopOne(c, q) || more;
  return more;
}

// ---------------------------------------------------------------------------
// Passive scalar transport (dbnsFoam calculateScalarTransport.H:1-384): a
// 1x0 coupled system for rhoS solved after the flow iterations
// ---------------------------------------------------------------------------
struct SMat {
  std::vector<double> diag, lower, upper;
  std::vector<double> iface;  // [B] coupled (cyclic) interface coefficients
};

void scalarBoundary(Case& c) {
  for (int b = 0; b < c.B; ++b) {
    const int pi = c.bpatch[b];
    c.sB[b] = c.sFixed[pi] ? c.sValue[pi] : c.s[c.bcell[b]];
    if (isCyc(c, b)) {  // coupled evaluate
      const int pc = c.bpartner[b];
      c.sB[b] = c.bw[b] * (c.s[c.bcell[b]] - c.s[pc]) + c.s[pc];
    }
  }
}

void smatMul(const Case& c, const SMat& A, const double* x, double* y) {
  for (int i = 0; i < c.N; ++i) y[i] = A.diag[i] * x[i];
  for (int fi = 0; fi < c.F; ++fi) {
    const int l = c.own[fi], u = c.nei[fi];
    y[u] += A.lower[fi] * x[l];
    y[l] += A.upper[fi] * x[u];
  }
  if (!A.iface.empty())
    for (int b = 0; b < c.B; ++b)
      if (isCyc(c, b)) y[c.bcell[b]] += A.iface[b] * x[c.bpartner[b]];
}

// lusgs.C:50-385 with one scalar equation, sequential in cell order
int smatPrecondition(const Case& c, const SMat& A, double* r) {
  if (c.cfg.preconditioner == ICS_PC_NONE) return ICS_OK;
  if (c.cfg.preconditioner == ICS_PC_JACOBI) {
    for (int i = 0; i < c.N; ++i) r[i] /= A.diag[i];
    return ICS_OK;
  }
  std::vector<double> rD(c.N);
  for (int i = 0; i < c.N; ++i) {
    rD[i] = 1.0 / std::max(1.0 / GREAT, std::fabs(A.diag[i]));
    if (rD[i] < VSMALL) return ICS_ERR_DIAG;
  }
  for (int ci = 0; ci < c.N; ++ci) {
    const double d = rD[ci] * r[ci];
    for (int fi : c.cellFaces[ci])
      if (c.own[fi] == ci && c.nei[fi] > ci) r[c.nei[fi]] -= A.lower[fi] * d;
  }
  for (int ci = c.N - 1; ci >= 0; --ci) {
    const double d = rD[ci] * r[ci];
    r[ci] = d;
    for (int fi : c.cellFaces[ci])
      if (c.nei[fi] == ci && c.own[fi] < ci) r[c.own[fi]] -= A.upper[fi] * d;
  }
  return ICS_OK;
}

// gmres::solveDelta for the 1x0 system (norm factor, MGS, Givens, restart)
int scalarGmres(Case& c, const SMat& A, const std::vector<double>& b, const std::vector<double>& w,
                std::vector<double>& dx, ics_solver_perf& perf) {
  const int N = c.N, m = c.cfg.n_directions;
  std::memset(&perf, 0, sizeof(perf));
  double avg = 0;
  for (int i = 0; i < N; ++i) avg += w[i];
  avg /= N;
  std::vector<double> wmr(N), tmp(N), r(b);
  for (int i = 0; i < N; ++i) wmr[i] = w[i] - avg;
  smatMul(c, A, wmr.data(), tmp.data());
  double nf = 0, sb = 0;
  for (int i = 0; i < N; ++i) {
    nf += std::fabs(tmp[i]) + std::fabs(b[i]);
    sb += std::fabs(b[i]);
  }
  nf += VSMALL;
  perf.init_res[0] = perf.final_res[0] = sb / nf;
  dx.assign(N, 0.0);
  std::vector<std::vector<double>> Vk(m, std::vector<double>(N));
  std::vector<double> H(m * m, 0.0), yh(m, 0.0), bh(m + 1, 0.0), cs(m, 0.0), sn(m, 0.0);
  auto givens = [](double h, double beta, double& cc, double& ss) {
    if (beta == 0) {
      cc = 1;
      ss = 0;
    } else if (std::fabs(beta) > std::fabs(h)) {
      const double tau = -h / beta;
      ss = 1.0 / std::sqrt(1.0 + sqr(tau));
      cc = ss * tau;
    } else {
      const double tau = -beta / h;
      cc = 1.0 / std::sqrt(1.0 + sqr(tau));
      ss = cc * tau;
    }
  };
  auto stop = [&]() {
    if (perf.n_iterations < c.cfg.min_iter) return false;
    const double rel = perf.final_res[0] / (perf.init_res[0] + ROOTVSMALL);
    return perf.n_iterations >= c.cfg.max_iter || perf.final_res[0] < c.cfg.tolerance || rel < c.cfg.rel_tol;
  };
  int status = ICS_OK;
  do {
    int st = smatPrecondition(c, A, r.data());
    if (st) {
      c.err = "All diagonals of the scalar matrix are zero";
      return st;
    }
    double beta = 0;
    for (int q = 0; q < N; ++q) beta += sqr(r[q]);
    beta = std::sqrt(beta);
    if (!(beta > 0) || !std::isfinite(beta)) {
      status = std::isfinite(beta) ? ICS_ERR_BREAKDOWN : ICS_ERR_NONFINITE;
      perf.n_iterations++;
      break;
    }
    std::fill(bh.begin(), bh.end(), 0.0);
    bh[0] = beta;
    for (int i = 0; i < m; ++i) {
      for (int q = 0; q < N; ++q) Vk[i][q] = r[q] / beta;
      smatMul(c, A, Vk[i].data(), r.data());
      smatPrecondition(c, A, r.data());
      for (int j = 0; j <= i; ++j) {
        double sdot = 0;
        for (int q = 0; q < N; ++q) sdot += r[q] * Vk[j][q];
        H[j * m + i] = sdot;
        for (int q = 0; q < N; ++q) r[q] -= H[j * m + i] * Vk[j][q];
      }
      beta = 0;
      for (int q = 0; q < N; ++q) beta += sqr(r[q]);
      beta = std::sqrt(beta);
      for (int j = 0; j < i; ++j) {
        const double Hji = H[j * m + i];
        H[j * m + i] = cs[j] * Hji - sn[j] * H[(j + 1) * m + i];
        H[(j + 1) * m + i] = sn[j] * Hji + cs[j] * H[(j + 1) * m + i];
      }
      givens(H[i * m + i], beta, cs[i], sn[i]);
      const double bhi = bh[i];
      bh[i] = cs[i] * bhi - sn[i] * bh[i + 1];
      bh[i + 1] = sn[i] * bhi + cs[i] * bh[i + 1];
      H[i * m + i] = cs[i] * H[i * m + i] - sn[i] * beta;
    }
    for (int i = m - 1; i >= 0; --i) {
      double sum = bh[i];
      for (int j = i + 1; j < m; ++j) sum -= H[i * m + j] * yh[j];
      const double hii = H[i * m + i];
      yh[i] = sum / (hii >= 0 ? hii + VSMALL : hii - VSMALL);
    }
    for (int i = 0; i < m; ++i)
      for (int q = 0; q < N; ++q) dx[q] += yh[i] * Vk[i][q];
    smatMul(c, A, dx.data(), r.data());
    double sr = 0;
    for (int q = 0; q < N; ++q) {
      r[q] = b[q] - r[q];
      sr += std::fabs(r[q]);
    }
    perf.final_res[0] = sr / nf;
    perf.n_iterations++;
  } while (!stop());
  perf.converged = status == ICS_OK;
  return status;
}

// one pass of calculateScalarTransport.H at the current flow state
int scalarTransportStep(Case& c, ics_solver_perf& perf) {
  const int N = c.N, F = c.F, B = c.B, NF = F + B;
  const std::vector<double> rhoSPrev = c.rhoS;
  VolS sF{c.s, c.sB};
  VolS rF = fieldRho(c);
  std::vector<double> s_l, s_r, rho_l, rho_r;
  std::vector<V3> U_l, U_r;
  reconstruct(c, sF, +1, c.reconS, s_l);
  reconstruct(c, sF, -1, c.reconS, s_r);
  reconstruct(c, rF, +1, c.cfg.recon_rho, rho_l);
  reconstruct(c, rF, -1, c.cfg.recon_rho, rho_r);
  reconstructU(c, +1, U_l);
  reconstructU(c, -1, U_r);
  // face flux phiSp: Roe-averaged upwinding with Harten's fix (lines 82-146)
  std::vector<double> phiS(NF);
  for (int fi = 0; fi < NF; ++fi) {
    const double ms = magSfOf(c, fi);
    const V3 n = SfOf(c, fi) / ms;
    const double rS_l = rho_l[fi] * s_l[fi], rS_r = rho_r[fi] * s_r[fi];
    const double coefR = std::sqrt(std::max(VSMALL, rho_r[fi]) / std::max(VSMALL, rho_l[fi]));
    const V3 roeU = (coefR * U_r[fi] + U_l[fi]) / (coefR + 1.0);
    const double um = umOf(c, fi);
    const double uProj = dot(roeU, n) - um;
    double lam = std::fabs(uProj);
    const double eps = 0.05 * lam;
    if (lam < eps) lam = (sqr(lam) + sqr(eps)) / (2.0 * eps);
    double ph = -0.5 * ms * lam * (rS_r - rS_l);
    ph += 0.5 * ms * (rho_l[fi] * dot(U_l[fi], n) * s_l[fi] + rho_r[fi] * dot(U_r[fi], n) * s_r[fi]);
    ph -= 0.5 * ms * um * (rS_l + rS_r);
    phiS[fi] = ph;
  }
  // residual -div(phiSp) [+ laplacian(D, s)] [- physical ddt]
  std::vector<double> div(N, 0.0), lap(N, 0.0);
  for (int fi = 0; fi < F; ++fi) {
    div[c.own[fi]] += phiS[fi];
    div[c.nei[fi]] -= phiS[fi];
  }
  for (int b = 0; b < B; ++b) div[c.bcell[b]] += phiS[F + b];
  const bool viscous = c.cfg.viscous != 0;
  if (viscous) {
    std::vector<V3> gs;
    gaussGrad(c, sF, gs);
    for (int fi = 0; fi < F; ++fi) {
      const int o = c.own[fi], nb = c.nei[fi];
      const double wf = c.w[fi];
      const V3 d = c.C[nb] - c.C[o];
      const V3 kcor = c.Sf[fi] / c.magSf[fi] - d * c.nodc[fi];
      const V3 gf(wf * (gs[o].x - gs[nb].x) + gs[nb].x, wf * (gs[o].y - gs[nb].y) + gs[nb].y,
                  wf * (gs[o].z - gs[nb].z) + gs[nb].z);
      const double sn = c.nodc[fi] * (c.s[nb] - c.s[o]) + dot(kcor, gf);
      const double lf = (c.Ds * c.magSf[fi]) * sn;
      lap[o] += lf;
      lap[nb] -= lf;
    }
    for (int b = 0; b < B; ++b) lap[c.bcell[b]] += (c.Ds * c.bmagSf[b]) * ((c.sB[b] - c.s[c.bcell[b]]) * c.bdc[b]);
  }
  const bool steady = c.cfg.ddt_scheme == ICS_DDT_STEADY;
  const DdtCoeffs dd = ddtCoeffs(c);
  std::vector<double> bsrc(N);
  for (int i = 0; i < N; ++i) {
    const double Vc = c.V[i];
    double r = -(div[i] / Vc);
    if (viscous) r += lap[i] / Vc;
    if (!steady) {
      double dg, sr;
      ddtMatrix(c, dd, i, c.rhoS[i], c.rhoS0[i], c.rhoS00[i], dg, sr);
      r -= (dg * c.rhoS[i] - sr) / Vc;
    }
    bsrc[i] = r * Vc;
  }
  // Jacobian (lines 197-343)
  SMat A;
  A.diag.assign(N, 0.0);
  A.lower.assign(F, 0.0);
  A.upper.assign(F, 0.0);
  for (int fi = 0; fi < F; ++fi) {
    const V3 n = c.Sf[fi] / c.magSf[fi];
    const double up = 0.5 * c.magSf[fi] * dot(U_r[fi], n);
    const double lo = -0.5 * c.magSf[fi] * dot(U_l[fi], n);
    A.upper[fi] += up;
    A.lower[fi] += lo;
    A.diag[c.own[fi]] -= lo;
    A.diag[c.nei[fi]] -= up;
  }
  // coupled (cyclic) faces: interface 0.5|S| U_r.n, diagonal -(-0.5|S| U_l.n)
  if (c.hasCyc) {
    A.iface.assign(B, 0.0);
    for (int b = 0; b < B; ++b) {
      if (!isCyc(c, b)) continue;
      const int fi = F + b;
      const V3 n = c.bSf[b] / c.bmagSf[b];
      const double up = 0.5 * c.bmagSf[b] * dot(U_r[fi], n);
      const double lo = -0.5 * c.bmagSf[b] * dot(U_l[fi], n);
      A.iface[b] += up;
      A.diag[c.bcell[b]] -= lo;
      if (c.mrfOn) {
        const double phm = c.mrfU[fi] * c.bmagSf[b];
        A.iface[b] -= phm * (1 - c.bw[b]);
        A.diag[c.bcell[b]] -= phm * c.bw[b];
      }
    }
  }
  // MRF: -div(w, u_MRF |S|) (lines 217-219)
  if (c.mrfOn)
    for (int fi = 0; fi < F; ++fi) {
      const double phm = c.mrfU[fi] * c.magSf[fi];
      const double up = phm * (1 - c.w[fi]), lo = -phm * c.w[fi];
      A.upper[fi] -= up;
      A.lower[fi] -= lo;
      A.diag[c.own[fi]] -= -lo;
      A.diag[c.nei[fi]] -= -up;
    }
  // dissipation with lambdaConv = |interpolate(U).n - u_MRF| (internal and boundary faces)
  for (int fi = 0; fi < F; ++fi) {
    const int o = c.own[fi], nb = c.nei[fi];
    const double wf = c.w[fi];
    const V3 Uf(wf * (c.U[o].x - c.U[nb].x) + c.U[nb].x, wf * (c.U[o].y - c.U[nb].y) + c.U[nb].y,
                wf * (c.U[o].z - c.U[nb].z) + c.U[nb].z);
    const double lc = std::fabs(dot(Uf, c.Sf[fi] / c.magSf[fi]) - umOf(c, fi));
    const double d = 0.5 * c.magSf[fi] * lc;
    A.upper[fi] -= d;
    A.lower[fi] -= d;
    A.diag[o] += d;
    A.diag[nb] += d;
  }
  for (int b = 0; b < B; ++b) {
    // (on a coupled face U_B is the interpolate of U with the partner rotated)
    const double lc = std::fabs(dot(c.UB[b], c.bSf[b] / c.bmagSf[b]) - umOf(c, F + b));
    A.diag[c.bcell[b]] += 0.5 * c.bmagSf[b] * lc;
    if (isCyc(c, b)) A.iface[b] -= 0.5 * c.bmagSf[b] * lc;
  }
  // geometric boundaries: rho_B (U_B . S_B) valueInternalCoeffs / rho_I
  for (int b = 0; b < B; ++b) {
    const int ci = c.bcell[b];
    if (isCyc(c, b)) continue;
    const double vic = c.sFixed[c.bpatch[b]] ? 0.0 : 1.0;
    const double flux = rhoBof(c, b) * (dot(c.UB[b], c.bSf[b]) - umOf(c, F + b) * c.bmagSf[b]) * vic;
    A.diag[ci] += flux * (1.0 / c.rho[ci]);
  }
  if (viscous) {
    for (int fi = 0; fi < F; ++fi) {
      const int o = c.own[fi], nb = c.nei[fi];
      const double rhof = c.w[fi] * (c.rho[o] - c.rho[nb]) + c.rho[nb];
      const double stab = 0.5 * (c.Ds / rhof) * c.magSf[fi] * c.dc[fi];
      A.upper[fi] -= stab;
      A.lower[fi] -= stab;
      A.diag[o] += stab;
      A.diag[nb] += stab;
    }
  }
  for (int i = 0; i < N; ++i) {
    double dg, sr;
    ddtMatrix(c, dd, i, c.rhoS[i], c.rhoS0[i], c.rhoS00[i], dg, sr);
    A.diag[i] += dg;
  }
  std::vector<double> dx;
  const int st = scalarGmres(c, A, bsrc, rhoSPrev, dx, perf);
  if (st && st != ICS_ERR_BREAKDOWN) return st;
  for (int i = 0; i < N; ++i) {
    c.rhoS[i] += dx[i];
    c.s[i] = c.rhoS[i] / c.rho[i];
  }
  scalarBoundary(c);
  return ICS_OK;
}

}  // namespace

struct ics_handle_s : Case {};

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void icsref_default_config(ics_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->R = 287.0;
  c->Cp = 1004.5;
  c->mu = 0;
  c->Pr = 0.72;
  c->As = 1.458e-6;
  c->Ts = 110.4;
  c->flux_scheme = ICS_FLUX_AUSMPLUSUP;
  c->low_mach_ausm = 1;
  c->entropy_fix_coeff = 0.05;
  c->recon_rho = c->recon_U = c->recon_T = ICS_RECON_UPWIND;
  c->ddt_scheme = ICS_DDT_STEADY;
  c->delta_t = 1;
  c->solver = ICS_SOLVER_GMRES;
  c->preconditioner = ICS_PC_LUSGS;
  c->n_directions = 8;
  c->max_iter = 1000;
  c->min_iter = 0;
  c->tolerance = 1e-12;
  c->rel_tol = 1e-2;
  c->precision = ICS_PREC_FP64;
  c->n_pseudo_corr = 20;
  c->n_pseudo_corr_min = 1;
  c->pseudo_tol = 1e-5;
  c->pseudo_tol_rel = 1e-5;
  c->pseudo_co_num = 1;
  c->pseudo_co_num_min = 0.1;
  c->pseudo_co_num_max = 25;
  c->pseudo_co_max_increase = 1.25;
  c->pseudo_co_min_decrease = 0.1;
  c->local_timestepping = 1;
  c->local_timestepping_bounding = 1;
  c->local_timestepping_lower_bound = 0.95;
  c->reset_pseudo = 0;
  c->rho_min = -GREAT;
  c->T_min = SMALL;
  c->T_max = GREAT;
  c->n_sweeps = 1;
  c->viscous_lf_jacobian = 1;
  c->limiter_coeff = 1.0;
}

int icsref_set_config(ics_handle h, const ics_config* cfg) {
  if (!h || !cfg) return ICS_ERR_ARG;
  if (cfg->flux_scheme < 0 || cfg->flux_scheme > 2) {
    h->err = "Unknown convectiveFluxScheme";
    return ICS_ERR_SCHEME;
  }
  if (cfg->preconditioner < 0 || cfg->preconditioner > 2 ||
      (cfg->solver != ICS_SOLVER_GMRES && cfg->solver != ICS_SOLVER_SMOOTH) || cfg->n_sweeps < 1) {
    h->err = "Unknown solver or preconditioner";
    return ICS_ERR_SCHEME;
  }
  if (cfg->viscous_lf_jacobian != 0 && cfg->viscous_lf_jacobian != 1) return ICS_ERR_ARG;
  if (!(cfg->limiter_coeff > 0.0 && cfg->limiter_coeff <= 1.0)) return ICS_ERR_ARG;
  if (cfg->n_directions < 1 || cfg->n_directions > 64) return ICS_ERR_ARG;
  if (h->nInst > 1 && (cfg->ddt_scheme != ICS_DDT_STEADY || cfg->solver != ICS_SOLVER_GMRES)) {
    h->err = "Harmonic Balance needs steadyState ddt and the GMRES solver";
    return ICS_ERR_ARG;
  }
  h->cfg = *cfg;
  h->Cv = cfg->Cp - cfg->R;
  h->gamma = cfg->Cp / h->Cv;
  if (!cfg->local_timestepping) {
    h->err = "global pseudo time stepping is not supported";
    return ICS_ERR_ARG;
  }
  return ICS_OK;
}

int icsref_create(const ics_mesh_desc* m, const ics_config* cfg, ics_handle* out) {
  if (!m || !cfg || !out || m->n_cells <= 0 || m->n_faces < 0 || m->n_bfaces < 0) return ICS_ERR_ARG;
  ics_handle h = new ics_handle_s();
  Case& c = *h;
  c.N = m->n_cells;
  c.Nc = c.N;
  c.F = m->n_faces;
  c.B = m->n_bfaces;
  c.own.assign(m->owner, m->owner + c.F);
  c.nei.assign(m->neighbour, m->neighbour + c.F);
  for (int f = 0; f < c.F; ++f) {
    if (c.own[f] < 0 || c.nei[f] >= c.N || c.own[f] >= c.nei[f]) {
      delete h;
      return ICS_ERR_ARG;
    }
  }
  c.Sf.resize(c.F);
  c.Cf.resize(c.F);
  c.magSf.resize(c.F);
  for (int f = 0; f < c.F; ++f) {
    c.Sf[f] = V3(m->Sf[3 * f], m->Sf[3 * f + 1], m->Sf[3 * f + 2]);
    c.Cf[f] = V3(m->Cf[3 * f], m->Cf[3 * f + 1], m->Cf[3 * f + 2]);
    c.magSf[f] = mag(c.Sf[f]);
  }
  c.w.assign(m->weights, m->weights + c.F);
  c.dc.assign(m->delta_coeffs, m->delta_coeffs + c.F);
  c.nodc.assign(m->nonorth_delta_coeffs, m->nonorth_delta_coeffs + c.F);
  c.C.resize(c.N);
  for (int i = 0; i < c.N; ++i) c.C[i] = V3(m->C[3 * i], m->C[3 * i + 1], m->C[3 * i + 2]);
  c.V.assign(m->V, m->V + c.N);
  c.bcell.assign(m->b_cell, m->b_cell + c.B);
  c.bpatch.assign(m->b_patch, m->b_patch + c.B);
  c.bSf.resize(c.B);
  c.bCf.resize(c.B);
  c.bmagSf.resize(c.B);
  for (int b = 0; b < c.B; ++b) {
    if (c.bcell[b] < 0 || c.bcell[b] >= c.N || c.bpatch[b] < 0 || c.bpatch[b] >= m->n_patches) {
      delete h;
      return ICS_ERR_ARG;
    }
    c.bSf[b] = V3(m->b_Sf[3 * b], m->b_Sf[3 * b + 1], m->b_Sf[3 * b + 2]);
    c.bCf[b] = V3(m->b_Cf[3 * b], m->b_Cf[3 * b + 1], m->b_Cf[3 * b + 2]);
    c.bmagSf[b] = mag(c.bSf[b]);
  }
  c.bdc.assign(m->b_delta_coeffs, m->b_delta_coeffs + c.B);
  for (int p = 0; p < m->n_patches; ++p) {
    const ics_patch_desc& d = m->patches[p];
    Patch q;
    q.kind = d.kind;
    q.is_wall = d.is_wall;
    q.p = d.p;
    q.T = d.T;
    for (int k = 0; k < 3; ++k) q.U[k] = d.U[k];
    q.p0 = d.p0;
    q.T0 = d.T0;
    for (int k = 0; k < 9; ++k) q.R[k] = d.rotation[k];
    if (d.kind == ICS_PATCH_CYCLIC) c.hasCyc = true;
    c.patches.push_back(q);
  }
  if (c.hasCyc) {
    if (!m->b_partner || !m->b_weights || !m->b_nbr_d) {
      delete h;
      return ICS_ERR_ARG;
    }
    c.bpartner.assign(c.B, -1);
    c.bw.assign(c.B, 1.0);
    c.bnodc.resize(c.B);
    c.bdelta.assign(c.B, V3());
    c.bnbrd.assign(c.B, V3());
    for (int b = 0; b < c.B; ++b) {
      c.bnodc[b] = m->b_nonorth_delta_coeffs ? m->b_nonorth_delta_coeffs[b] : m->b_delta_coeffs[b];
      if (c.patches[c.bpatch[b]].kind != ICS_PATCH_CYCLIC) continue;
      c.bpartner[b] = m->b_partner[b];
      c.bw[b] = m->b_weights[b];
      c.bnbrd[b] = V3(m->b_nbr_d[3 * b], m->b_nbr_d[3 * b + 1], m->b_nbr_d[3 * b + 2]);
      c.bdelta[b] = (c.bCf[b] - c.C[c.bcell[b]]) - c.bnbrd[b];
    }
  }
  for (int k = 0; k < 3; ++k) c.solD[k] = m->solution_d[k];
  c.cellFaces.assign(c.N, {});
  for (int f = 0; f < c.F; ++f) c.cellFaces[c.own[f]].push_back(f);
  for (int f = 0; f < c.F; ++f) c.cellFaces[c.nei[f]].push_back(f);
  int st = icsref_set_config(h, cfg);
  if (st) {
    delete h;
    return st;
  }
  const int N = c.N;
  c.rho.assign(N, 0);
  c.rhoE.assign(N, 0);
  c.p.assign(N, 0);
  c.T.assign(N, 0);
  c.e.assign(N, 0);
  c.rhoU.assign(N, V3());
  c.U.assign(N, V3());
  c.pB.assign(c.B, 0);
  c.TB.assign(c.B, 0);
  c.phiB.assign(c.B, 0);
  c.UB.assign(c.B, V3());
  c.pseudoCo.assign(N, cfg->pseudo_co_num);
  c.rPseudoDeltaT.assign(N, 0.0);
  c.ddtCoeff.assign(N, 0.0);
  *out = h;
  return ICS_OK;
}

int icsref_destroy(ics_handle h) {
  delete h;
  return ICS_OK;
}

int icsref_last_error(ics_handle h, char* buf, int32_t len) {
  if (!h || !buf || len <= 0) return ICS_ERR_ARG;
  std::snprintf(buf, len, "%s", h->err.c_str());
  return ICS_OK;
}

static void copyOld(Case& c) {
  c.rho0 = c.rho;
  c.rhoE0 = c.rhoE;
  c.rhoU0 = c.rhoU;
  c.rho00 = c.rho;
  c.rhoE00 = c.rhoE;
  c.rhoU00 = c.rhoU;
}

int icsref_set_primitive(ics_handle h, const double* p, const double* U, const double* T) {
  if (!h || !p || !U || !T) return ICS_ERR_ARG;
  Case& c = *h;
  for (int i = 0; i < c.N; ++i) {
    c.p[i] = p[i];
    c.T[i] = T[i];
    c.U[i] = V3(U[3 * i], U[3 * i + 1], U[3 * i + 2]);
    c.e[i] = heOf(c, c.T[i]);
    c.rho[i] = psiOf(c, c.T[i]) * c.p[i];
    c.rhoU[i] = c.rho[i] * c.U[i];
    c.rhoE[i] = c.rho[i] * (c.e[i] + 0.5 * magSqr(c.U[i]));
  }
  // boundary initial guess: interior values, then one BC evaluation
  std::vector<double> psiB(c.B);
  for (int b = 0; b < c.B; ++b) {
    const int ci = c.bcell[b];
    c.pB[b] = c.p[ci];
    c.TB[b] = c.T[ci];
    c.UB[b] = c.U[ci];
    c.phiB[b] = psiOf(c, c.TB[b]) * c.pB[b] * dot(c.UB[b], c.bSf[b]);
    psiB[b] = psiOf(c, c.TB[b]);
  }
  correctBoundaryConditions(c, psiB);
  copyOld(c);
  c.timeIndex = 0;
  return ICS_OK;
}

int icsref_set_boundary_state(ics_handle h, const double* pb, const double* Ub, const double* Tb, const double* phib) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  for (int b = 0; b < c.B; ++b) {
    if (pb) c.pB[b] = pb[b];
    if (Tb) c.TB[b] = Tb[b];
    if (Ub) c.UB[b] = V3(Ub[3 * b], Ub[3 * b + 1], Ub[3 * b + 2]);
    if (phib) c.phiB[b] = phib[b];
  }
  return ICS_OK;
}

int icsref_get_boundary_state(ics_handle h, double* pb, double* Ub, double* Tb, double* phib) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  for (int b = 0; b < c.B; ++b) {
    if (pb) pb[b] = c.pB[b];
    if (Tb) Tb[b] = c.TB[b];
    if (Ub)
      for (int k = 0; k < 3; ++k) Ub[3 * b + k] = c.UB[b][k];
    if (phib) phib[b] = c.phiB[b];
  }
  return ICS_OK;
}

int icsref_get_state(ics_handle h, double* W, double* p, double* U, double* T) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  for (int i = 0; i < c.N; ++i) {
    if (W) {
      W[5 * i] = c.rho[i];
      W[5 * i + 1] = c.rhoU[i].x;
      W[5 * i + 2] = c.rhoU[i].y;
      W[5 * i + 3] = c.rhoU[i].z;
      W[5 * i + 4] = c.rhoE[i];
    }
    if (p) p[i] = c.p[i];
    if (T) T[i] = c.T[i];
    if (U)
      for (int k = 0; k < 3; ++k) U[3 * i + k] = c.U[i][k];
  }
  return ICS_OK;
}

int icsref_set_conservative(ics_handle h, const double* W, int32_t set_old) {
  if (!h || !W) return ICS_ERR_ARG;
  Case& c = *h;
  for (int i = 0; i < c.N; ++i) {
    c.rho[i] = W[5 * i];
    c.rhoU[i] = V3(W[5 * i + 1], W[5 * i + 2], W[5 * i + 3]);
    c.rhoE[i] = W[5 * i + 4];
    c.U[i] = c.rhoU[i] / c.rho[i];
    c.e[i] = c.rhoE[i] / c.rho[i] - 0.5 * magSqr(c.U[i]);
    c.T[i] = c.e[i] / c.Cv;
    c.p[i] = c.rho[i] / psiOf(c, c.T[i]);
  }
  if (set_old) copyOld(c);
  return ICS_OK;
}

int icsref_set_pseudo_co(ics_handle h, const double* co) {
  if (!h || !co) return ICS_ERR_ARG;
  h->pseudoCo.assign(co, co + h->N);
  return ICS_OK;
}

int icsref_get_pseudo_co(ics_handle h, double* co, double* rdt) {
  if (!h) return ICS_ERR_ARG;
  for (int i = 0; i < h->N; ++i) {
    if (co) co[i] = h->pseudoCo[i];
    if (rdt) rdt[i] = h->rPseudoDeltaT[i];
  }
  return ICS_OK;
}

int icsref_calc_flux(ics_handle h, double* phi, double* phiU, double* phiE) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  calcFlux(c);
  const int NF = c.F + c.B;
  for (int f = 0; f < NF; ++f) {
    if (phi) phi[f] = c.phi[f];
    if (phiE) phiE[f] = c.phiE[f];
    if (phiU)
      for (int k = 0; k < 3; ++k) phiU[3 * f + k] = c.phiU[f][k];
  }
  return ICS_OK;
}

int icsref_residual(ics_handle h, double* source) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  calcFlux(c);
  residualSource(c);
  setCoAndDeltaT(c);
  if (source) std::memcpy(source, c.src.data(), sizeof(double) * 5 * c.N);
  for (double v : c.src)
    if (!std::isfinite(v)) {
      c.err = "non-finite residual";
      return ICS_ERR_NONFINITE;
    }
  return ICS_OK;
}

int icsref_assemble_jacobian(ics_handle h) {
  if (!h) return ICS_ERR_ARG;
  assembleJacobian(*h);
  return ICS_OK;
}

int icsref_get_jacobian(ics_handle h, double* diag, double* lower, double* upper) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  if (!c.haveMatrix) return ICS_ERR_STATE;
  for (int i = 0; i < c.N; ++i)
    if (diag) std::memcpy(diag + 25 * i, c.diag[i].a, sizeof(double) * 25);
  for (int f = 0; f < c.F; ++f) {
    if (lower) std::memcpy(lower + 25 * f, c.lower[f].a, sizeof(double) * 25);
    if (upper) std::memcpy(upper + 25 * f, c.upper[f].a, sizeof(double) * 25);
  }
  return ICS_OK;
}

int icsref_matrix_mul(ics_handle h, const double* x, double* y) {
  if (!h || !x || !y) return ICS_ERR_ARG;
  if (!h->haveMatrix) return ICS_ERR_STATE;
  matrixMul(*h, x, y);
  return ICS_OK;
}

int icsref_precondition(ics_handle h, double* r) {
  if (!h || !r) return ICS_ERR_ARG;
  Case& c = *h;
  if (!c.haveMatrix) return ICS_ERR_STATE;
  std::vector<double> rD;
  if (c.cfg.preconditioner == ICS_PC_LUSGS && !lusgsDiag(c, rD)) return ICS_ERR_DIAG;
  return precondition(c, rD, r);
}

int icsref_solve_increment(ics_handle h, ics_solver_perf* perf, double* dW) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  if (!c.haveMatrix) return ICS_ERR_STATE;
  storeW(c, c.Wprev);
  ResIO rio;
  int st = c.cfg.solver == ICS_SOLVER_SMOOTH ? smoothSolveDelta(c, c.Wprev, rio, c.dW)
                                             : gmresSolveDelta(c, c.Wprev, rio, c.dW);
  c.haveIncrement = true;
  ics_solver_perf pf;
  toPerf(rio, pf);
  pf.converged = st == ICS_OK;
  if (perf) *perf = pf;
  if (dW) std::memcpy(dW, c.dW.data(), sizeof(double) * 5 * c.N);
  c.initRes = rio.init;
  c.initResValid = true;
  for (int J = 0; J < c.nInst; ++J) std::memcpy(c.ctl[J].residuals, &rio.init[5 * J], 5 * sizeof(double));
  return st;
}

int icsref_update_fields(ics_handle h, ics_iter_stats* st) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  if (!c.haveIncrement) return ICS_ERR_STATE;
  boundLocalTimeStep(c);
  int bounded = 0;
  int s = updateFields(c, c.dW, bounded);
  c.haveIncrement = false;
  if (st) {
    st->bounded_cells = bounded;
    st->rho_l2_residual = c.lastRhoL2;
  }
  return s;
}

int icsref_pseudo_iteration(ics_handle h, ics_iter_stats* st) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  ics_iter_stats s{};
  int r = icsref_residual(h, nullptr);
  if (r) return r;
  assembleJacobian(c);
  r = icsref_solve_increment(h, &s.perf, nullptr);
  if (r && r != ICS_ERR_BREAKDOWN) return r;
  int bounded = 0;
  boundLocalTimeStep(c);
  int u = updateFields(c, c.dW, bounded);
  c.haveIncrement = false;
  s.bounded_cells = bounded;
  s.rho_l2_residual = c.lastRhoL2;
  double m = 0;
  for (int i = 0; i < c.N; ++i) m += c.pseudoCo[i];
  s.pseudo_co_mean = m / c.N;
  s.status = r ? r : u;
  if (st) *st = s;
  return u;
}

int icsref_begin_time_step(ics_handle h) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  const bool steady = c.cfg.ddt_scheme == ICS_DDT_STEADY;
  // runTime++: old-old <- old <- current
  c.rho00 = c.rho0;
  c.rhoU00 = c.rhoU0;
  c.rhoE00 = c.rhoE0;
  c.rho0 = c.rho;
  c.rhoU0 = c.rhoU;
  c.rhoE0 = c.rhoE;
  if (c.timeIndex == 0) {
    c.rho00 = c.rho0;
    c.rhoU00 = c.rhoU0;
    c.rhoE00 = c.rhoE0;
  }
  if (c.scalarOn) {
    c.rhoS00 = c.timeIndex == 0 ? c.rhoS : c.rhoS0;
    c.rhoS0 = c.rhoS;
  }
  mrfBoundaryVelocity(c);  // outerLoop.H:6
  c.timeIndex++;
  if (!steady) {
    c.initResValid = false;
    c.prevResValid = false;
  }
  if (c.cfg.reset_pseudo) std::fill(c.pseudoCo.begin(), c.pseudoCo.end(), c.cfg.pseudo_co_num);
  return ICS_OK;
}

// phase-lag cyclic patches (the same arrays as ics_set_phase_lag); mode == NULL switches them off
int icsref_set_phase_lag(ics_handle h, const int32_t* mode, const double* P) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  c.plagMode.clear();
  c.plagP.clear();
  if (!mode) return ICS_OK;
  const int np = (int)c.patches.size(), n = c.nInst;
  if (n < 2 || !P) return ICS_ERR_ARG;
  for (int p = 0; p < np; ++p)
    if (mode[p] < 0 || mode[p] > 2 || (mode[p] && c.patches[p].kind != ICS_PATCH_CYCLIC)) return ICS_ERR_ARG;
  c.plagMode.assign(mode, mode + np);
  c.plagP.assign(P, P + (size_t)np * n * n);
  return ICS_OK;
}

// MRF zones (the same arrays as ics_set_mrf); omega == NULL switches them off
int icsref_set_mrf(ics_handle h, const double* omega, const double* face_velocity, const double* boundary_U,
                   const int32_t* included, int32_t mode) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  c.mrfOn = false;
  c.mrfU.clear();
  c.mrfOm.clear();
  c.mrfBU.clear();
  c.mrfBIn.clear();
  c.haveMatrix = c.haveIncrement = false;
  if (!omega) return ICS_OK;
  if (!face_velocity || (c.B > 0 && (!boundary_U || !included)) ||
      (mode != ICS_MRF_OUTER_LOOP && mode != ICS_MRF_EVERY_UPDATE))
    return ICS_ERR_ARG;
  c.mrfU.assign(face_velocity, face_velocity + c.F + c.B);
  c.mrfOm.resize(c.N);
  for (int i = 0; i < c.N; ++i) c.mrfOm[i] = V3(omega[3 * i], omega[3 * i + 1], omega[3 * i + 2]);
  c.mrfBU.resize(c.B);
  c.mrfBIn.resize(c.B);
  for (int b = 0; b < c.B; ++b) {
    c.mrfBU[b] = V3(boundary_U[3 * b], boundary_U[3 * b + 1], boundary_U[3 * b + 2]);
    c.mrfBIn[b] = included[b];
  }
  c.mrfEvery = mode == ICS_MRF_EVERY_UPDATE;
  c.mrfOn = true;
  mrfBoundaryVelocity(c);  // createFields.H:262-263
  return ICS_OK;
}

// Harmonic Balance: the handle's cells are n_instances stacked copies of one
// mesh (instance-major); D is the row-major n x n spectral operator
int icsref_set_hb(ics_handle h, int32_t n, const double* D) {
  if (!h || n < 1 || n > ICS_MAX_INSTANCES || (n > 1 && !D)) return ICS_ERR_ARG;
  Case& c = *h;
  if (c.N % n != 0) {
    c.err = "cell count is not a multiple of the number of instances";
    return ICS_ERR_ARG;
  }
  if (n > 1 && (c.cfg.ddt_scheme != ICS_DDT_STEADY || c.cfg.solver != ICS_SOLVER_GMRES)) {
    c.err = "Harmonic Balance needs steadyState ddt and the GMRES solver";
    return ICS_ERR_ARG;
  }
  for (int q = 0; q < n * n && n > 1; ++q)
    if (!std::isfinite(D[q])) return ICS_ERR_ARG;
  c.nInst = n;
  c.Nc = c.N / n;
  c.Dhb.assign(n > 1 ? D : nullptr, n > 1 ? D + n * n : nullptr);
  c.hbZone.clear();
  c.hbCyl = false;
  c.ctl.assign(n, Case::Control());
  c.initResValid = c.prevResValid = false;
  c.haveMatrix = c.haveIncrement = false;
  return ICS_OK;
}

int icsref_set_hb_zone(ics_handle h, const int32_t* zone, int32_t cyl_coords, const double axis[3],
                       const double origin[3]) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  if (c.nInst < 2) return ICS_ERR_ARG;
  c.hbZone.clear();
  if (zone) {
    c.hbZone.resize(c.N);
    for (int i = 0; i < c.N; ++i) c.hbZone[i] = zone[i % c.Nc] != 0;
  }
  c.hbCyl = cyl_coords != 0;
  if (c.hbCyl) {
    if (!axis || !origin) return ICS_ERR_ARG;
    const V3 a(axis[0], axis[1], axis[2]);
    const double ma = std::sqrt(dot(a, a));
    if (!(ma > 0)) return ICS_ERR_ARG;
    c.hbAxis = a / ma;
    c.hbOrigin = V3(origin[0], origin[1], origin[2]);
  }
  c.haveMatrix = c.haveIncrement = false;
  return ICS_OK;
}

int icsref_scalar_enable(ics_handle h, const double* s, const int32_t* patch_fixed, const double* patch_value,
                         double D, int32_t recon) {
  if (!h || !s || recon < 0 || recon > ICS_RECON_MUSCL_MINMOD || D < 0) return ICS_ERR_ARG;
  Case& c = *h;
  if (c.hasCyc && c.cfg.viscous) return ICS_ERR_ARG;  // the scalar's laplacian across cyclic patches is not built
  if (c.nInst > 1) {
    c.err = "scalar transport is not provided for Harmonic Balance handles";
    return ICS_ERR_ARG;
  }
  const int P = (int)c.patches.size();
  c.sFixed.assign(P, 0);
  c.sValue.assign(P, 0.0);
  for (int p = 0; p < P; ++p) {
    c.sFixed[p] = patch_fixed ? (patch_fixed[p] != 0) : 0;
    c.sValue[p] = patch_value ? patch_value[p] : 0.0;
  }
  c.s.assign(s, s + c.N);
  c.sB.assign(c.B, 0.0);
  c.rhoS.resize(c.N);
  for (int i = 0; i < c.N; ++i) c.rhoS[i] = c.rho[i] * c.s[i];
  c.rhoS0 = c.rhoS;
  c.rhoS00 = c.rhoS;
  c.Ds = D;
  c.reconS = recon;
  scalarBoundary(c);
  c.scalarOn = true;
  return ICS_OK;
}

int icsref_scalar_transport(ics_handle h, int32_t n_iterations, ics_solver_perf* perf) {
  if (!h || n_iterations < 0) return ICS_ERR_ARG;
  Case& c = *h;
  if (!c.scalarOn) {
    c.err = "scalar transport is not enabled";
    return ICS_ERR_STATE;
  }
  ics_solver_perf pf{};
  for (int it = 0; it < n_iterations; ++it) {
    const int st = scalarTransportStep(c, pf);
    if (st) return st;
  }
  if (perf) *perf = pf;
  return ICS_OK;
}

int icsref_get_scalar(ics_handle h, double* s, double* rhoS) {
  if (!h) return ICS_ERR_ARG;
  Case& c = *h;
  if (!c.scalarOn) return ICS_ERR_STATE;
  if (s) std::memcpy(s, c.s.data(), sizeof(double) * c.N);
  if (rhoS) std::memcpy(rhoS, c.rhoS.data(), sizeof(double) * c.N);
  return ICS_OK;
}

int icsref_pseudo_loop(ics_handle h, int32_t* more) {
  if (!h || !more) return ICS_ERR_ARG;
  *more = pseudoLoop(*h) ? 1 : 0;
  return ICS_OK;
}

}  // extern "C"
