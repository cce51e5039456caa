// Pieces of the residual pipeline shared by its kernels (k_residual.cu) and
// the reverse-mode derivative of the residual (k_adjoint.cu): scheme
// parameters, the reconstruction of a face value, and the host helpers that
// fill them from a handle.
#pragma once

#include <type_traits>

#include "flux.cuh"
#include "hb.cuh"
#include "ics_internal.cuh"

namespace ics {

template <typename Real>
constexpr bool is_fp64 = std::is_same<Real, double>::value;

struct ResParams {
  double R, Cv, gamma, cstarFac;
  int scheme, reconRho, reconU, reconT, lowMach;
  double entropyFix;
};

__device__ __forceinline__ int recon_of(const ResParams& P, int q) {
  if (q == Q_RHO || q == Q_P) return P.reconRho;
  if (q == Q_UX || q == Q_UY || q == Q_UZ) return P.reconU;
  return P.reconT;
}

// TVD limitedScheme face value from the two cell values and the upwind
// cell's gradient projected on C_nei - C_own (NVD/TVD r with vanLeer or Minmod)
template <typename Real, typename GT>
__device__ __forceinline__ Real tvd_face(int scheme, double wf, double wUp, const Real& qo, const Real& qn,
                                         const GT& gradcf) {
  const Real gradf = qn - qo;
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
  const Real wgt = lim * wf + (1.0 - lim) * wUp;
  return wgt * (qo - qn) + qn;
}

// reconstruct field k on face f for direction dir (+1 owner side, -1 neighbour side)
template <typename Real>
__device__ __forceinline__ Real reconstruct(const DevMesh& m, int scheme, int k, int f, int o, int nb, const Real& qo,
                                            const Real& qn, const Real* __restrict__ grad, double dir) {
  const int N = m.N, F = m.F;
  const double wUp = dir > 0 ? 1.0 : 0.0;
  if (scheme == ICS_RECON_UPWIND) return wUp * (qo - qn) + qn;
  if (scheme == ICS_RECON_VANLEER || scheme == ICS_RECON_MINMOD) {
    const int c = dir > 0 ? o : nb;
    const double d0 = m.dCC[f], d1 = m.dCC[F + f], d2 = m.dCC[2 * F + f];
    const Real gradcf = d0 * grad[(3 * k) * N + c] + d1 * grad[(3 * k + 1) * N + c] + d2 * grad[(3 * k + 2) * N + c];
    return tvd_face(scheme, m.w[f], wUp, qo, qn, gradcf);
  }
  // MUSCL: upwind value + limited-gradient extrapolation; the neighbour
  // side's upwind value 0 (qo - qn) + qn is qn itself
  const int c = dir > 0 ? o : nb;
  const double* d = dir > 0 ? m.dOwn : m.dNei;
  const Real base = dir > 0 ? (qo - qn) + qn : qn;
  return base + (d[f] * grad[(3 * k) * N + c] + d[F + f] * grad[(3 * k + 1) * N + c] +
                 d[2 * F + f] * grad[(3 * k + 2) * N + c]);
}

ResParams res_params(const Handle& h);
// fields with a reconstruction gradient (bit k = q field k) and the limiter
// kind of the MUSCL groups (0 none, 1 minmod, 2 Venkatakrishnan)
unsigned grad_mask(const Handle& h, int* limited);

}  // namespace ics
