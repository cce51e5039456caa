// Harmonic Balance source coupling of one cell (HBZone::addSource,
// HBZone.C:359-652, HBZoneTemplates.C:39-92): the source of instance J's cell
// is -V sum_K D_JK W_K over the same cell of every instance K, for the cells
// of the HB zone only; with cylCoords the momentum of each instance is taken
// in cylindrical components (radial, circumferential, axial) about the zone's
// axis at that instance's cell centre, combined with D and turned back into
// Cartesian components at instance J's cell centre.
#pragma once

#include "ics_internal.cuh"

namespace ics {

__device__ __forceinline__ bool hb_in_zone(const DevMesh& m, int c) { return !m.hbZone || m.hbZone[c]; }

// radial and circumferential unit vectors of the cylindrical frame at cell c
__device__ __forceinline__ void hb_frame(const DevMesh& m, int c, double rh[3], double th[3]) {
  const int N = m.N;
  const double* a = m.hbAxis;
  double r[3] = {m.C[c] - m.hbOrigin[0], m.C[N + c] - m.hbOrigin[1], m.C[2 * N + c] - m.hbOrigin[2]};
  const double ar = a[0] * r[0] + a[1] * r[1] + a[2] * r[2];
  for (int k = 0; k < 3; ++k) r[k] -= ar * a[k];
  const double mr = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  for (int k = 0; k < 3; ++k) rh[k] = r[k] / mr;
  th[0] = a[1] * rh[2] - a[2] * rh[1];
  th[1] = a[2] * rh[0] - a[0] * rh[2];
  th[2] = a[0] * rh[1] - a[1] * rh[0];
}

// out[k] += coef * sum_K D_JK x_K[k] for the cell c of instance J (x a
// cell-major [N][5] field, Real double or Dual); momentum through the
// cylindrical frames when m.hbCyl; nothing outside the zone
template <typename Real, typename XT>
__device__ __forceinline__ void hb_apply(const DevMesh& m, int c, double coef, const XT* x, Real out[5]) {
  if (!hb_in_zone(m, c)) return;
  const int n = m.nInst, J = c / m.Nc, cl = c - J * m.Nc;
  Real s[5] = {Real(0.0), Real(0.0), Real(0.0), Real(0.0), Real(0.0)};
  for (int K = 0; K < n; ++K) {
    const int ck = K * m.Nc + cl;
    const double d = coef * m.Dhb[J * n + K];
    const XT* xk = x + 5 * (size_t)ck;
    s[0] = s[0] + d * xk[0];
    s[4] = s[4] + d * xk[4];
    if (m.hbCyl) {
      double rh[3], th[3];
      hb_frame(m, ck, rh, th);
      const double* a = m.hbAxis;
      s[1] = s[1] + d * (xk[1] * rh[0] + xk[2] * rh[1] + xk[3] * rh[2]);
      s[2] = s[2] + d * (xk[1] * th[0] + xk[2] * th[1] + xk[3] * th[2]);
      s[3] = s[3] + d * (xk[1] * a[0] + xk[2] * a[1] + xk[3] * a[2]);
    } else {
      for (int k = 1; k < 4; ++k) s[k] = s[k] + d * xk[k];
    }
  }
  out[0] = out[0] + s[0];
  out[4] = out[4] + s[4];
  if (m.hbCyl) {
    double rh[3], th[3];
    hb_frame(m, c, rh, th);
    const double* a = m.hbAxis;
    for (int k = 0; k < 3; ++k) out[1 + k] = out[1 + k] + s[1] * rh[k] + s[2] * th[k] + s[3] * a[k];
  } else {
    for (int k = 1; k < 4; ++k) out[k] = out[k] + s[k];
  }
}

// the transpose of hb_apply, gathered at cell c of instance K:
// out += coef * sum_J D_JK T_K^T T_J u_J over the zone
__device__ __forceinline__ void hb_apply_transpose(const DevMesh& m, int c, double coef, const double* u,
                                                   double out[5]) {
  if (!hb_in_zone(m, c)) return;
  const int n = m.nInst, K = c / m.Nc, cl = c - K * m.Nc;
  double s[5] = {0, 0, 0, 0, 0};
  for (int J = 0; J < n; ++J) {
    const int cj = J * m.Nc + cl;
    const double d = coef * m.Dhb[J * n + K];
    const double* uj = u + 5 * (size_t)cj;
    s[0] += d * uj[0];
    s[4] += d * uj[4];
    if (m.hbCyl) {  // the cylindrical components of u_J at instance J's centre
      double rh[3], th[3];
      hb_frame(m, cj, rh, th);
      const double* a = m.hbAxis;
      s[1] += d * (uj[1] * rh[0] + uj[2] * rh[1] + uj[3] * rh[2]);
      s[2] += d * (uj[1] * th[0] + uj[2] * th[1] + uj[3] * th[2]);
      s[3] += d * (uj[1] * a[0] + uj[2] * a[1] + uj[3] * a[2]);
    } else {
      for (int k = 1; k < 4; ++k) s[k] += d * uj[k];
    }
  }
  out[0] += s[0];
  out[4] += s[4];
  if (m.hbCyl) {  // back to Cartesian components at instance K's centre
    double rh[3], th[3];
    hb_frame(m, c, rh, th);
    const double* a = m.hbAxis;
    for (int k = 0; k < 3; ++k) out[1 + k] += s[1] * rh[k] + s[2] * th[k] + s[3] * a[k];
  } else {
    for (int k = 1; k < 4; ++k) out[k] += s[k];
  }
}

}  // namespace ics
