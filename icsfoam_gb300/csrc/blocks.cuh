// Off-diagonal blocks of the sliced-ELL Jacobian: factored in FP32 storage,
// full 5x5 in FP64 storage.
//
// Every off-diagonal block the reference inserts for an internal face is a
// convective flux Jacobian of one side's state times +-0.5|S| plus multiples
// of the identity (blockFvMatrix::insertBlock / insertDissipationBlock,
// blockFvMatrix.C:211-326; the MRF term -div(w, u_MRF |S|) and the LF viscous
// laplacian, convectiveFluxScheme.C:467-482, viscousFluxScheme.C:234-247):
//     upper_f = A(W_R, 0.5|S| n) + c0 I,   lower_f = A(W_L, -0.5|S| n) + c0 I
// where A(W, s) is the Euler flux Jacobian of state (U, E) for the (scaled)
// normal s -- every entry of A is linear in s.  A slot therefore stores
// eight words, s (3), U (3), E, c0, instead of 25, and the products apply
// A(U, E, s) x in closed form: 32 B per FP32 slot instead of 100 B for the
// HBM-bound Krylov kernels, for about 45 flops per product.  In FP64 those
// flops would run on GB300's slow FP64 pipe and make the kernels ALU-bound,
// so FP64 storage keeps the 25 entries (SlotBlock<double>).
//
// The viscous Jacobian without LaxFriedrichJacobian (viscousFluxScheme.C:
// 249-267) adds minus the five laplacians at the column cell to each slot:
// the two face coefficients (mu_f|S|)dc, (alpha_f|S|)dc per slot (vjslot,
// [slot][2][32]) and the column cell's -U/rho (3), 1/rho, -E/rho + |U|^2/rho
// (vjcell, [5][N]) are stored beside and applied by vj_sub.
#pragma once

#include "ics_internal.cuh"

namespace ics {

template <typename TB>
struct SlotBlock;

// words per stored slot: 8 factored (FP32), 25 full (FP64)
inline int slot_words(bool fp32) { return fp32 ? 8 : 25; }

template <>
struct SlotBlock<double> {
  static constexpr int W = 25;
  double w[W];
  __device__ __forceinline__ void load(const double* __restrict__ blk, size_t slot, int lane) {
    const double* p = blk + slot * W * 32 + lane;
#pragma unroll
    for (int q = 0; q < W; ++q) w[q] = p[q * 32];
  }
  template <typename TV>
  __device__ __forceinline__ void mv(TV, const TV* x, TV* y) const {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      TV a = TV(0);
#pragma unroll
      for (int j = 0; j < 5; ++j) a += TV(w[5 * i + j]) * x[j];
      y[i] = a;
    }
  }
  template <typename TV>
  __device__ __forceinline__ void mv2(TV g, const TV* xa, TV* ya, const TV* xb, TV* yb) const {
    mv(g, xa, ya);
    mv(g, xb, yb);
  }
  __device__ __forceinline__ double entry(double, int i, int j) const { return w[5 * i + j]; }
};

template <>
struct SlotBlock<float> {
  using TB = float;
  static constexpr int W = 8;
  TB w[W];  // s0 s1 s2 U0 U1 U2 E c0

  __device__ __forceinline__ void load(const TB* __restrict__ blk, size_t slot, int lane) {
    const TB* p = blk + slot * W * 32 + lane;
#pragma unroll
    for (int q = 0; q < W; ++q) w[q] = p[q * 32];
  }

  // y = B x
  template <typename TV>
  __device__ __forceinline__ void mv(TV g, const TV* x, TV* y) const {
    Terms<TV> t(g, w);
    t.apply(g, x, y);
  }
  // ya = B xa, yb = B xb with the per-block terms computed once
  template <typename TV>
  __device__ __forceinline__ void mv2(TV g, const TV* xa, TV* ya, const TV* xb, TV* yb) const {
    Terms<TV> t(g, w);
    t.apply(g, xa, ya);
    t.apply(g, xb, yb);
  }

  // entry (i, j) of the convective part (matrix readback)
  __device__ __forceinline__ double entry(double g, int i, int j) const {
    const double S[3] = {double(w[0]), double(w[1]), double(w[2])};
    const double U[3] = {double(w[3]), double(w[4]), double(w[5])};
    const double a2 = g - 1.0;
    const double th = 0.5 * a2 * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
    const double a1 = g * double(w[6]) - th;
    const double pu = U[0] * S[0] + U[1] * S[1] + U[2] * S[2];
    double e;
    if (i == 0) {
      e = (j == 0 || j == 4) ? 0.0 : S[j - 1];
    } else if (i == 4) {
      e = j == 0 ? pu * (th - a1) : (j == 4 ? g * pu : S[j - 1] * a1 - a2 * U[j - 1] * pu);
    } else {
      const int r = i - 1;
      if (j == 0)
        e = S[r] * th - U[r] * pu;
      else if (j == 4)
        e = S[r] * a2;
      else
        e = U[r] * S[j - 1] - a2 * S[r] * U[j - 1] + (r == j - 1 ? pu : 0.0);
    }
    if (i == j) e += double(w[7]);
    return e;
  }

 private:
  template <typename TV>
  struct Terms {
    TV a2, S0, S1, S2, U0, U1, U2, th, a1, pu, c;
    __device__ __forceinline__ Terms(TV g, const TB* w) {
      a2 = g - TV(1);
      S0 = TV(w[0]);
      S1 = TV(w[1]);
      S2 = TV(w[2]);
      U0 = TV(w[3]);
      U1 = TV(w[4]);
      U2 = TV(w[5]);
      th = TV(0.5) * a2 * (U0 * U0 + U1 * U1 + U2 * U2);
      a1 = g * TV(w[6]) - th;
      pu = U0 * S0 + U1 * S1 + U2 * S2;
      c = TV(w[7]);
    }
    __device__ __forceinline__ void apply(TV g, const TV* x, TV* y) const {
      const TV x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3], x4 = x[4];
      const TV sx = S0 * x1 + S1 * x2 + S2 * x3;
      const TV ux = U0 * x1 + U1 * x2 + U2 * x3;
      const TV t1 = th * x0 - a2 * ux + a2 * x4;  // multiplies s_r in rows 1-3
      const TV t2 = sx - pu * x0;                 // multiplies U_r in rows 1-3
      const TV d = pu + c;
      y[0] = sx + c * x0;
      y[1] = S0 * t1 + U0 * t2 + d * x1;
      y[2] = S1 * t1 + U1 * t2 + d * x2;
      y[3] = S2 * t1 + U2 * t2 + d * x3;
      y[4] = pu * (th - a1) * x0 + a1 * sx - a2 * pu * ux + (g * pu + c) * x4;
    }
  };
};

// y -= V x, V = the non-LF viscous laplacians at column cell col of slot
// (only when m.vjslot is set; TB is the block storage type)
template <typename TB, typename TV>
__device__ __forceinline__ void vj_sub(const DevMesh& m, size_t slot, int lane, int col, const TV* x, TV* y) {
  const TB* vs = (const TB*)m.vjslot + slot * 2 * 32 + lane;
  const TB* vc = (const TB*)m.vjcell;
  const int N = m.N;
  const TV mg = TV(vs[0]), ag = TV(vs[32]);
  const TV m0 = TV(vc[col]), m1 = TV(vc[N + col]), m2 = TV(vc[2 * N + col]);
  const TV ir = TV(vc[3 * N + col]), eR = TV(vc[4 * N + col]);
  y[1] -= mg * (m0 * x[0] + ir * x[1]);
  y[2] -= mg * (m1 * x[0] + ir * x[2]);
  y[3] -= mg * (m2 * x[0] + ir * x[3]);
  y[4] -= ag * (eR * x[0] + m0 * x[1] + m1 * x[2] + m2 * x[3] + ir * x[4]);
}

// entry (i, j) of V (matrix readback)
template <typename TB>
__device__ __forceinline__ double vj_entry(const DevMesh& m, size_t slot, int lane, int col, int i, int j) {
  const TB* vs = (const TB*)m.vjslot + slot * 2 * 32 + lane;
  const TB* vc = (const TB*)m.vjcell;
  const int N = m.N;
  const double mg = double(vs[0]), ag = double(vs[32]);
  const double mU[3] = {double(vc[col]), double(vc[N + col]), double(vc[2 * N + col])};
  const double ir = double(vc[3 * N + col]), eR = double(vc[4 * N + col]);
  if (i >= 1 && i <= 3) {
    if (j == 0) return mU[i - 1] * mg;
    if (j == i) return ir * mg;
    return 0.0;
  }
  if (i == 4) return j == 0 ? eR * ag : (j == 4 ? ir * ag : mU[j - 1] * ag);
  return 0.0;
}

}  // namespace ics
