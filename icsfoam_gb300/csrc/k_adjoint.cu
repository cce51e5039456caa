// Reverse-mode derivative of the residual source: u -> (d(R V)/dW)^T u.
//
// The residual is a chain of local maps, each of which the backward pass
// transposes in reverse order, recomputing what it needs from the state
// instead of storing the forward pass or any Jacobian:
//
//   W --(cell)--> q --(Gauss gradient + cellLimited limiter)--> g
//     --(face: reconstruction + flux)--> F --(cell: -div)--> R V
//
//   1. recompute q and the limited gradients g at the current state (the
//      forward kernels of the residual, k_fields and k_grad);
//   2. k_adj_face (internal faces): F_bar = u_nei - u_own, then the adjoints
//      of the two reconstructed face states, F_bar . dF/dq_L and
//      F_bar . dF/dq_R, with the flux's local partial derivatives taken by
//      forward-mode dual numbers through the same flux function the residual
//      uses (16 inputs, 5 outputs; one pass per input);
//   3. k_adj_lim (cells): the reconstruction's transpose (the upwind value
//      and the gradient extrapolation d . g of every face of the cell), then
//      the transpose of the cellLimited limiter, recomputing the cell's Gauss
//      gradient, its bounds and which neighbour / face set them: it yields
//      the adjoint of the cell's unlimited gradient and of the values the
//      limiter read (the cell's own, and the neighbour that attained the
//      bound, recorded for the next pass);
//   4. k_adj_cell (cells): the Gauss gradient's transpose (each face value
//      w q_own + (1 - w) q_nei feeds both cells' gradients), the recorded
//      bound contributions of the neighbours, and the transpose of the
//      pointwise map W -> q (five dual-number passes of the cell map), plus
//      the diagonal physical ddt, MRF rotation and Harmonic Balance terms.
//
// Every branch (limiter selection, flux region) is decided on the values as
// the forward pass decides it, so this is the transpose of ics_jvp's linear
// map exactly (to round-off).  Boundary values are held fixed, as there.
// For the TVD limitedScheme reconstructions (vanLeer, Minmod) the face value
// depends on both cells and on the upwind cell's unlimited gradient: the face
// kernel transposes it there and hands on the adjoint of the gradient's
// projection.  Not provided (the entry point returns ICS_ERR_ARG): viscous
// terms and cyclic patches.
#include "residual.cuh"

namespace ics {

// Pointwise map W -> q of one cell: the primitives of k_derive (U = rhoU /
// rho, e = rhoE / rho - |U|^2 / 2, T = e / Cv, p = rho R T) then the fields
// of k_fields (E, H, sound speed or AUSM+up's c*), in the same arithmetic.
template <typename Real>
__device__ __forceinline__ void cell_q(const Real W[5], const ResParams& P, Real q[NQ]) {
  const Real rho = W[0];
  const Real U[3] = {W[1] / rho, W[2] / rho, W[3] / rho};
  const Real e = W[4] / rho - 0.5 * dot3(U, U);
  const Real T = e / P.Cv;
  const Real p = rho / (1.0 / (P.R * T));
  const Real E = P.Cv * T + 0.5 * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
  const Real H = fmax(E, SMALL) + fmax(p / rho, SMALL);
  const Real psi = 1.0 / (P.R * T);
  const Real cl = sqrt(P.gamma / psi);
  q[Q_RHO] = rho;
  q[Q_P] = p;
  q[Q_UX] = U[0];
  q[Q_UY] = U[1];
  q[Q_UZ] = U[2];
  q[Q_E] = E;
  q[Q_H] = H;
  q[Q_C] = P.scheme == ICS_FLUX_AUSMPLUSUP ? sqrt(P.cstarFac * H) : fmax(cl, VSMALL);
}

// adjoint of the reconstructed face states: aF[j][F], j < NQ the owner-side
// (left) field j, j >= NQ the neighbour-side (right) field j - NQ
template <bool MRF>
__global__ void __launch_bounds__(128) k_adj_face(DevMesh m, ResParams P, const double* __restrict__ q,
                                                  const double* __restrict__ grad, const double* __restrict__ u,
                                                  double* __restrict__ aF, double* __restrict__ aS) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.F) return;
  const int N = m.N, F = m.F;
  const int o = m.own[f], nb = m.nei[f];
  double qs[2 * NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    if (P.scheme == ICS_FLUX_ROE && k == Q_C) {
      qs[k] = qs[NQ + k] = 0.0;
      continue;
    }
    const double qo = q[k * N + o], qn = q[k * N + nb];
    const int sch = recon_of(P, k);
    qs[k] = reconstruct(m, sch, k, f, o, nb, qo, qn, grad, +1.0);
    qs[NQ + k] = reconstruct(m, sch, k, f, o, nb, qo, qn, grad, -1.0);
  }
  double Fb[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) Fb[i] = u[5 * nb + i] - u[5 * o + i];
  const double n[3] = {m.nf[f], m.nf[F + f], m.nf[2 * F + f]};
  const double S[3] = {m.Sf[f], m.Sf[F + f], m.Sf[2 * F + f]};
  const double magS = m.magSf[f];
  const double um = MRF ? m.mrfU[f] : 0.0;
  double qb[2 * NQ];
#pragma unroll 1
  for (int j = 0; j < 2 * NQ; ++j) {
    if (P.scheme == ICS_FLUX_ROE && (j % NQ) == Q_C) {
      qb[j] = 0.0;
      continue;
    }
    Dual x[2 * NQ];
#pragma unroll
    for (int i = 0; i < 2 * NQ; ++i) x[i] = Dual(qs[i], i == j ? 1.0 : 0.0);
    FStateT<Dual> L{x[Q_RHO], x[Q_P], {x[Q_UX], x[Q_UY], x[Q_UZ]}, x[Q_E], x[Q_H], x[Q_C]};
    FStateT<Dual> R{x[NQ + Q_RHO], x[NQ + Q_P], {x[NQ + Q_UX], x[NQ + Q_UY], x[NQ + Q_UZ]},
                    x[NQ + Q_E],   x[NQ + Q_H], x[NQ + Q_C]};
    Dual out[5];
    if (P.scheme == ICS_FLUX_AUSMPLUSUP)
      flux_ausm(L, R, S, magS, P.lowMach, um, out);
    else if (P.scheme == ICS_FLUX_HLLC)
      flux_hllc(L, R, n, magS, P.gamma, um, out);
    else
      flux_roe(L, R, n, magS, P.gamma, P.entropyFix, um, out);
    double a = 0.0;
#pragma unroll
    for (int i = 0; i < 5; ++i) a += Fb[i] * out[i].d;
    qb[j] = a;
  }
  // the reconstructions' transpose: adjoints reaching the owner's and the
  // neighbour's value (aF[k], aF[NQ + k]); for the TVD limitedSchemes, whose
  // face value depends on both cells and on the upwind cell's gradient
  // projected on C_nei - C_own, also the adjoints of those projections of
  // the left and right values (aS[k], aS[NQ + k])
#pragma unroll 1
  for (int k = 0; k < NQ; ++k) {
    const int sch = recon_of(P, k);
    double ao = qb[k], an = qb[NQ + k], sl = 0.0, sr = 0.0;
    const bool used = !(P.scheme == ICS_FLUX_ROE && k == Q_C);  // Roe reconstructs no sound speed
    if (used && (sch == ICS_RECON_VANLEER || sch == ICS_RECON_MINMOD)) {
      const double qo = q[k * N + o], qn = q[k * N + nb];
      const double d0 = m.dCC[f], d1 = m.dCC[F + f], d2 = m.dCC[2 * F + f];
      const double gl = d0 * grad[(3 * k) * N + o] + d1 * grad[(3 * k + 1) * N + o] + d2 * grad[(3 * k + 2) * N + o];
      const double gr = d0 * grad[(3 * k) * N + nb] + d1 * grad[(3 * k + 1) * N + nb] +
                        d2 * grad[(3 * k + 2) * N + nb];
      const double wf = m.w[f];
      double dl[3], dr[3];  // d(value)/d(qo, qn, projected gradient)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const Dual xo(qo, i == 0 ? 1.0 : 0.0), xn(qn, i == 1 ? 1.0 : 0.0);
        dl[i] = tvd_face(sch, wf, 1.0, xo, xn, Dual(gl, i == 2 ? 1.0 : 0.0)).d;
        dr[i] = tvd_face(sch, wf, 0.0, xo, xn, Dual(gr, i == 2 ? 1.0 : 0.0)).d;
      }
      ao = qb[k] * dl[0] + qb[NQ + k] * dr[0];
      an = qb[k] * dl[1] + qb[NQ + k] * dr[1];
      sl = qb[k] * dl[2];
      sr = qb[NQ + k] * dr[2];
    }
    aF[(size_t)k * F + f] = ao;
    aF[(size_t)(NQ + k) * F + f] = an;
    aS[(size_t)k * F + f] = sl;
    aS[(size_t)(NQ + k) * F + f] = sr;
  }
}

// Per cell and field: the transpose of the reconstruction (upwind value and
// gradient extrapolation on every face of the cell) and of the cellLimited
// limiter.  Outputs: aQ[k][N] the adjoint reaching q_k of the cell directly,
// aG[3k+d][N] the adjoint of its unlimited Gauss gradient, and per bound
// (max: slot k, min: slot NQ + k) the neighbour cell that attained it
// (aSrc, -1 for none) and the adjoint it receives (aVal).
template <int LIMITED>
__global__ void __launch_bounds__(128) k_adj_lim(DevMesh m, unsigned mask, unsigned tvd,
                                                 const double* __restrict__ q, const double* __restrict__ bq,
                                                 const double* __restrict__ aF, const double* __restrict__ aS,
                                                 double* __restrict__ aQ, double* __restrict__ aG,
                                                 int* __restrict__ aSrc, double* __restrict__ aVal) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int N = m.N, F = m.F, B = m.B;
  const int e0 = m.cptr[c], e1 = m.cptr[c + 1];
  const int b0 = m.bptr[c], b1 = m.bptr[c + 1];
#pragma unroll 1
  for (int k = 0; k < NQ; ++k) {
    const bool hasGrad = (mask >> k) & 1;
    double qd = 0.0, gb[3] = {0.0, 0.0, 0.0};
    for (int e = e0; e < e1; ++e) {
      const int code = m.cface[e];
      const bool isOwn = code >= 0;
      const int f = isOwn ? code : ~code;
      const double a = aF[(size_t)(isOwn ? k : NQ + k) * F + f];
      qd += a;
      if (hasGrad && ((tvd >> k) & 1)) {  // TVD: the upwind gradient's projection on C_nei - C_own
        const double sa = aS[(size_t)(isOwn ? k : NQ + k) * F + f];
        gb[0] += sa * m.dCC[f];
        gb[1] += sa * m.dCC[F + f];
        gb[2] += sa * m.dCC[2 * F + f];
      } else if (hasGrad) {  // linearUpwind: the extrapolation d . g from the cell to the face
        const double* d = isOwn ? m.dOwn : m.dNei;
        gb[0] += a * d[f];
        gb[1] += a * d[F + f];
        gb[2] += a * d[2 * F + f];
      }
    }
    int sMax = -1, sMin = -1;
    double vMax = 0.0, vMin = 0.0;
    if (hasGrad && LIMITED) {
      // recompute the Gauss gradient and the bounds exactly as k_grad does
      const double qc = q[k * N + c];
      double G[3] = {0.0, 0.0, 0.0};
      double qmax = qc, qmin = qc;
      int srcMax = c, srcMin = c;  // -1: a boundary value
      for (int e = e0; e < e1; ++e) {
        const int code = m.cface[e];
        const bool isOwn = code >= 0;
        const int f = isOwn ? code : ~code;
        const int other = isOwn ? m.nei[f] : m.own[f];
        const double wf = m.w[f];
        const double sg = isOwn ? 1.0 : -1.0;
        const double S0 = sg * m.Sf[f], S1 = sg * m.Sf[F + f], S2 = sg * m.Sf[2 * F + f];
        const double qo = q[k * N + other];
        const double qown = isOwn ? qc : qo, qnei = isOwn ? qo : qc;
        const double sf = wf * (qown - qnei) + qnei;
        G[0] = G[0] + S0 * sf;
        G[1] = G[1] + S1 * sf;
        G[2] = G[2] + S2 * sf;
        if (okey(qo) > okey(qmax)) {
          qmax = qo;
          srcMax = other;
        }
        if (okey(qo) < okey(qmin)) {
          qmin = qo;
          srcMin = other;
        }
      }
      for (int e = b0; e < b1; ++e) {
        const int b = m.bface[e];
        const double v = bq[k * B + b];
        G[0] = G[0] + m.bSf[b] * v;
        G[1] = G[1] + m.bSf[B + b] * v;
        G[2] = G[2] + m.bSf[2 * B + b] * v;
        if (okey(v) > okey(qmax)) {
          qmax = v;
          srcMax = -1;
        }
        if (okey(v) < okey(qmin)) {
          qmin = v;
          srcMin = -1;
        }
      }
      const double rV = 1.0 / m.V[c];
      G[0] = G[0] * rV;
      G[1] = G[1] * rV;
      G[2] = G[2] * rV;
      double dmax = qmax - qc, dmin = qmin - qc;
      if (m.limWiden > 0.0) {
        const double wd = m.limWiden * (dmax - dmin);
        dmax = dmax + wd;
        dmin = dmin - wd;
      }
      // the largest positive / most negative face extrapolation and its d
      double epos = 0.0, eneg = 0.0, dpos[3] = {0, 0, 0}, dneg[3] = {0, 0, 0};
      bool small = false;
      auto faceExtrap = [&](double d0, double d1, double d2) {
        const double ex = d0 * G[0] + d1 * G[1] + d2 * G[2];
        if (ogt(ex, SMALL)) {
          if (okey(ex) > okey(epos)) {
            epos = ex;
            dpos[0] = d0, dpos[1] = d1, dpos[2] = d2;
          }
        } else if (olt(ex, -SMALL)) {
          if (okey(ex) < okey(eneg)) {
            eneg = ex;
            dneg[0] = d0, dneg[1] = d1, dneg[2] = d2;
          }
        } else {
          small = true;
        }
      };
      for (int e = e0; e < e1; ++e) {
        const int code = m.cface[e];
        const bool isOwn = code >= 0;
        const int f = isOwn ? code : ~code;
        const double* d = isOwn ? m.dOwn : m.dNei;
        faceExtrap(d[f], d[F + f], d[2 * F + f]);
      }
      for (int e = b0; e < b1; ++e) {
        const int b = m.bface[e];
        faceExtrap(m.bdOwn[b], m.bdOwn[B + b], m.bdOwn[2 * B + b]);
      }
      // the selection of k_grad: 0 none, 1 max bound / e+, 2 min bound / e-, 3 the r = 1 of a small face
      int sel = 0;
      double ra = 1.0, rb = 1.0;
      if (epos > 0.0) {
        ra = dmax;
        rb = epos;
        sel = 1;
      }
      if (eneg < 0.0) {
        const double a2 = -dmin, b2 = -eneg;
        if (sel == 0 || a2 * rb < ra * b2) {
          ra = a2;
          rb = b2;
          sel = 2;
        }
      }
      if (small && (sel == 0 || ra > rb)) {
        ra = 1.0;
        rb = 1.0;
        sel = 3;
      }
      const bool anyFace = (e1 > e0) || (b1 > b0);
      double lim = 1.0, lr = 1.0, dra = 0.0, drb = 0.0;
      if (anyFace && sel != 0) {
        if (LIMITED == 2) {
          const double num = ra * ra + 2 * ra * rb, den = ra * ra + ra * rb + 2 * rb * rb;
          lr = num / den;
          dra = ((2 * ra + 2 * rb) * den - num * (2 * ra + rb)) / (den * den);
          drb = (2 * ra * den - num * (ra + 4 * rb)) / (den * den);
        } else {
          lr = ra / rb;
          dra = 1.0 / rb;
          drb = -ra / (rb * rb);
        }
        lim = fmin(1.0, lr);
      }
      // g = lim G: G_bar = lim g_bar + (limiter terms), lim_bar = g_bar . G
      const double limBar = gb[0] * G[0] + gb[1] * G[1] + gb[2] * G[2];
      gb[0] *= lim;
      gb[1] *= lim;
      gb[2] *= lim;
      if (anyFace && (sel == 1 || sel == 2) && !(1.0 <= lr)) {
        const double raBar = limBar * dra, rbBar = limBar * drb;
        double dmaxBar = 0.0, dminBar = 0.0;
        if (sel == 1) {
          dmaxBar = raBar;
          gb[0] += rbBar * dpos[0];
          gb[1] += rbBar * dpos[1];
          gb[2] += rbBar * dpos[2];
        } else {
          dminBar = -raBar;
          gb[0] -= rbBar * dneg[0];
          gb[1] -= rbBar * dneg[1];
          gb[2] -= rbBar * dneg[2];
        }
        if (m.limWiden > 0.0) {
          const double w = m.limWiden;
          const double a = (1.0 + w) * dmaxBar - w * dminBar, b = -w * dmaxBar + (1.0 + w) * dminBar;
          dmaxBar = a;
          dminBar = b;
        }
        // d = bound - q_c: the cell's own value, and the bound's source
        qd -= dmaxBar + dminBar;
        if (srcMax == c) qd += dmaxBar;
        else if (srcMax >= 0) sMax = srcMax, vMax = dmaxBar;
        if (srcMin == c) qd += dminBar;
        else if (srcMin >= 0) sMin = srcMin, vMin = dminBar;
      }
    }
    aQ[(size_t)k * N + c] = qd;
    aG[(size_t)(3 * k) * N + c] = hasGrad ? gb[0] : 0.0;
    aG[(size_t)(3 * k + 1) * N + c] = hasGrad ? gb[1] : 0.0;
    aG[(size_t)(3 * k + 2) * N + c] = hasGrad ? gb[2] : 0.0;
    aSrc[(size_t)k * N + c] = sMax;
    aVal[(size_t)k * N + c] = vMax;
    aSrc[(size_t)(NQ + k) * N + c] = sMin;
    aVal[(size_t)(NQ + k) * N + c] = vMin;
  }
}

// Per cell: the Gauss gradient's transpose, the bound contributions the
// neighbours recorded, and the transpose of the cell map W -> q; plus the
// diagonal terms of the residual source (physical ddt, MRF rotation) and
// the Harmonic Balance coupling.
__global__ void __launch_bounds__(128) k_adj_cell(DevMesh m, ResParams P, unsigned mask, int limited,
                                                  double dgPhys, const double* __restrict__ W,
                                                  const double* __restrict__ aQ, const double* __restrict__ aG,
                                                  const int* __restrict__ aSrc, const double* __restrict__ aVal,
                                                  const double* __restrict__ u, double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int N = m.N, F = m.F;
  const int e0 = m.cptr[c], e1 = m.cptr[c + 1];
  double qb[NQ];
#pragma unroll 1
  for (int k = 0; k < NQ; ++k) {
    double acc = aQ[(size_t)k * N + c];
    if ((mask >> k) & 1) {
      for (int e = e0; e < e1; ++e) {
        const int code = m.cface[e];
        const bool isOwn = code >= 0;
        const int f = isOwn ? code : ~code;
        const int o = m.own[f], nb = m.nei[f];
        const double S0 = m.Sf[f], S1 = m.Sf[F + f], S2 = m.Sf[2 * F + f];
        const double go = S0 * aG[(size_t)(3 * k) * N + o] + S1 * aG[(size_t)(3 * k + 1) * N + o] +
                          S2 * aG[(size_t)(3 * k + 2) * N + o];
        const double gn = S0 * aG[(size_t)(3 * k) * N + nb] + S1 * aG[(size_t)(3 * k + 1) * N + nb] +
                          S2 * aG[(size_t)(3 * k + 2) * N + nb];
        const double sfBar = go / m.V[o] - gn / m.V[nb];
        const double wf = m.w[f];
        acc += (isOwn ? wf : 1.0 - wf) * sfBar;
        if (limited) {
          const int other = isOwn ? nb : o;
          if (aSrc[(size_t)k * N + other] == c) acc += aVal[(size_t)k * N + other];
          if (aSrc[(size_t)(NQ + k) * N + other] == c) acc += aVal[(size_t)(NQ + k) * N + other];
        }
      }
    }
    qb[k] = acc;
  }
  double r[5];
#pragma unroll 1
  for (int j = 0; j < 5; ++j) {
    Dual Wd[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) Wd[i] = Dual(W[5 * c + i], i == j ? 1.0 : 0.0);
    Dual qd[NQ];
    cell_q(Wd, P, qd);
    double a = 0.0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) a += qb[k] * qd[k].d;
    r[j] = a;
  }
  const double Vc = m.V[c];
#pragma unroll
  for (int k = 0; k < 5; ++k) r[k] -= dgPhys * Vc * u[5 * c + k];
  if (m.mrfOm) {  // u . (omega x v) = v . (u x omega)
    const double om[3] = {m.mrfOm[c], m.mrfOm[N + c], m.mrfOm[2 * N + c]};
    const double uU[3] = {u[5 * c + 1], u[5 * c + 2], u[5 * c + 3]};
    double cr[3];
    cross3(uU, om, cr);
#pragma unroll
    for (int k = 0; k < 3; ++k) r[1 + k] -= cr[k] * Vc;
  }
  if (m.nInst > 1) hb_apply_transpose(m, c, -Vc, u, r);  // -V_c sum_J D_JK u_(J,c) into instance K
#pragma unroll
  for (int k = 0; k < 5; ++k) out[5 * c + k] = r[k];
}

// ------------------------------------------------------------------ launch
static void ensure_adjoint(Handle& h) {
  if (h.aF) return;
  const size_t N = h.m.N, F = h.m.F;
  auto dal = [&](size_t bytes) {
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) throw CudaError(e, "cudaMalloc", __FILE__, __LINE__);
    return p;
  };
  h.aF = (double*)dal(2 * NQ * F * sizeof(double));
  h.aS = (double*)dal(2 * NQ * F * sizeof(double));
  h.aQ = (double*)dal(NQ * N * sizeof(double));
  h.aG = (double*)dal(3 * NQ * N * sizeof(double));
  h.aSrc = (int*)dal(2 * NQ * N * sizeof(int));
  h.aVal = (double*)dal(2 * NQ * N * sizeof(double));
}

std::string residual_vjp_unsupported(const Handle& h) {
  if (h.cfg.c.viscous) return "the reverse-mode residual derivative does not cover viscous terms";
  if (h.m.ncyc > 0) return "the reverse-mode residual derivative does not cover cyclic patches";
  return "";
}

void launch_residual_vjp(Handle& h, const double* u, double* out) {
  const std::string why = residual_vjp_unsupported(h);
  if (!why.empty()) throw why;
  ensure_adjoint(h);
  const ResParams P = res_params(h);
  // recompute the forward fields and limited gradients at this state
  launch_fields(h);
  launch_grad(h);
  int limited = 0;
  const unsigned mask = grad_mask(h, &limited);
  // fields reconstructed by a TVD limitedScheme (their gradient is unlimited)
  unsigned tvd = 0;
  for (int k = 0; k < NQ; ++k) {
    const int sch = k == Q_RHO || k == Q_P ? h.cfg.c.recon_rho
                                           : (k >= Q_UX && k <= Q_UZ ? h.cfg.c.recon_U : h.cfg.c.recon_T);
    if (sch == ICS_RECON_VANLEER || sch == ICS_RECON_MINMOD) tvd |= 1u << k;
  }
  if (h.m.F > 0) {
    if (h.m.mrfU)
      ICS_LAUNCH(h, ICS_K_ADJOINT, (k_adj_face<true><<<grid_for(h.m.F, 128), 128, 0, h.stream>>>(
                                       h.m, P, h.q, h.grad, u, h.aF, h.aS)));
    else
      ICS_LAUNCH(h, ICS_K_ADJOINT, (k_adj_face<false><<<grid_for(h.m.F, 128), 128, 0, h.stream>>>(
                                       h.m, P, h.q, h.grad, u, h.aF, h.aS)));
  }
  const int N = h.m.N;
  if (limited == 2)
    ICS_LAUNCH(h, ICS_K_ADJOINT, k_adj_lim<2><<<grid_for(N, 128), 128, 0, h.stream>>>(
                                     h.m, mask, tvd, h.q, h.bq, h.aF, h.aS, h.aQ, h.aG, h.aSrc, h.aVal));
  else if (limited == 1)
    ICS_LAUNCH(h, ICS_K_ADJOINT, k_adj_lim<1><<<grid_for(N, 128), 128, 0, h.stream>>>(
                                     h.m, mask, tvd, h.q, h.bq, h.aF, h.aS, h.aQ, h.aG, h.aSrc, h.aVal));
  else
    ICS_LAUNCH(h, ICS_K_ADJOINT, k_adj_lim<0><<<grid_for(N, 128), 128, 0, h.stream>>>(
                                     h.m, mask, tvd, h.q, h.bq, h.aF, h.aS, h.aQ, h.aG, h.aSrc, h.aVal));
  double dgPhys = 0.0;
  if (h.cfg.c.ddt_scheme == ICS_DDT_EULER) dgPhys = 1.0 / h.cfg.c.delta_t;
  if (h.cfg.c.ddt_scheme == ICS_DDT_BACKWARD) {
    const double dt = h.cfg.c.delta_t;
    const double dt0 = h.timeIndex <= 1 ? GREAT : dt;
    dgPhys = (1 + dt / (dt + dt0)) / dt;
  }
  ICS_LAUNCH(h, ICS_K_ADJOINT, k_adj_cell<<<grid_for(N, 128), 128, 0, h.stream>>>(
                                   h.m, P, mask, limited, dgPhys, h.W, h.aQ, h.aG, h.aSrc, h.aVal, u, out));
  ICS_CUDA(cudaGetLastError());
}

}  // namespace ics
