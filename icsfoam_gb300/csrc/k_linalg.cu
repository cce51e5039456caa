// Block linear algebra on the sliced-ELL Jacobian and the Krylov solver.
//
//   spmv      y = A x, thread per row; diagonal + one 5x5 block per face slot,
//             slots in column order (= face order, the order Amul adds them)
//   lusgs     (D_s + L) D_s^-1 (D_s + U) z = r with the scalar diagonal D_s,
//             level-scheduled: a level holds rows whose lower (forward) or
//             upper (reverse) neighbours all lie in earlier levels.  Within a
//             row the neighbour contributions are subtracted in the order the
//             sequential sweep of lusgs.C:233-384 applies them.
//   jacobi    z = D^-1 r with precomputed 5x5 inverses (Jacobi.C:55-135)
//   gmres     left-preconditioned restarted GMRES with modified Gram-Schmidt
//             and Givens rotations (gmres.C:772-1107).  All vectors and the
//             Hessenberg matrix stay on the device; dot products use a fixed
//             grid and a last-block-done tree, so results are reproducible
//             run to run.  One host synchronisation per restart cycle reads
//             the L1 residuals for the stop test (coupledMatrixSolver.C:198-221).
#include <algorithm>
#include <cmath>

#include "blocks.cuh"
#include "hb.cuh"
#include "ics_internal.cuh"

namespace ics {

// ------------------------------------------------------------------ reduce
// Returns true on the one thread (thread 0 of the last block) that wrote out[].
template <int NV>
__device__ __forceinline__ bool reduce_finish(double (&v)[NV], double* __restrict__ partials,
                                              unsigned int* __restrict__ counter, double* __restrict__ out) {
  __shared__ double sm[32][NV];
  __shared__ bool amLast;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sm[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int k = 0; k < NV; ++k) {
      double s = 0;
      for (int w = 0; w < nw; ++w) s += sm[w][k];
      partials[blockIdx.x * NV + k] = s;
    }
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    amLast = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (amLast) {  // block-uniform: the last block folds all partials in a fixed order
    __threadfence();
    const volatile double* vp = partials;
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] += vp[b * NV + k];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = acc[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) sm[warp][k] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int nw = blockDim.x >> 5;
      for (int k = 0; k < NV; ++k) {
        double s = 0;
        for (int w = 0; w < nw; ++w) s += sm[w][k];
        out[k] = s;
      }
      *counter = 0;
      return true;
    }
  }
  return false;
}

constexpr int RB = 256;  // threads per reduction block

// MGS steps stream 3 Krylov vectors of which two are L2-resident, so they are
// bound by latency and the reduction tail rather than by HBM: 4 blocks per SM
// (608 on 152 SMs) measured 11% faster than 8 per SM (sweep of 304-1216);
// the default of Handle::tuneMgsBlocks, which the autotuner may change.
constexpr int MGS_CHUNKS = 2;

// 16-byte vector of the Krylov element type
template <typename TV>
struct V16;
template <>
struct V16<float> {
  using T = float4;
  static constexpr int n = 4;
  __device__ static float get(const T& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
};
template <>
struct V16<double> {
  using T = double2;
  static constexpr int n = 2;
  __device__ static double get(const T& v, int k) { return k == 0 ? v.x : v.y; }
};

__device__ __forceinline__ void axpy16(float4& x, float h, const float4& p) {
  x.x -= h * p.x;
  x.y -= h * p.y;
  x.z -= h * p.z;
  x.w -= h * p.w;
}
__device__ __forceinline__ void axpy16(double2& x, double h, const double2& p) {
  x.x -= h * p.x;
  x.y -= h * p.y;
}
// Per-thread dot accumulation stays in the Krylov element type (a thread
// sums a few dozen products); FP64 conversions on GB300 run on the slow
// FP64 pipe, so the FP32 path converts once per thread, not per product.
__device__ __forceinline__ float dot16(const float4& a, const float4& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}
__device__ __forceinline__ double dot16(const double2& a, const double2& b) { return a.x * b.x + a.y * b.y; }

// ------------------------------------------------------------------- spmv
template <typename TB, typename TV>
__global__ void __launch_bounds__(128) k_spmv(DevMesh m, const TB* __restrict__ blk, const TB* __restrict__ dg,
                                              const TV* __restrict__ x, TV* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int s = c >> 5, lane = c & 31;
  TV xc[5], acc[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) xc[k] = x[5 * c + k];
  const TB* D = dg + (size_t)s * 25 * 32 + lane;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    TV a = TV(0);
#pragma unroll
    for (int j = 0; j < 5; ++j) a += TV(D[(5 * i + j) * 32]) * xc[j];
    acc[i] = a;
  }
  const int base = m.slot_base[s];
  const int ns = m.nslot[c];
  const TV g = TV(m.gamma);
#pragma unroll 1
  for (int t = 0; t < ns; ++t) {
    const int col = m.scol[(base + t) * 32 + lane];
    TV xj[5], y[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xj[k] = x[5 * col + k];
    SlotBlock<TB> Bk;
    Bk.load(blk, base + t, lane);
    Bk.mv(g, xj, y);
    if (m.vjslot) vj_sub<TB>(m, base + t, lane, col, xj, y);
#pragma unroll
    for (int i = 0; i < 5; ++i) acc[i] += y[i];
  }
  if (m.nInst > 1 && hb_in_zone(m, c)) {
    // Harmonic Balance coupling blocks V D_JK I with the other instances
    const int J = c / m.Nc, cl = c - J * m.Nc;
    const double Vc = m.V[c];
    for (int K = 0; K < m.nInst; ++K) {
      if (K == J) continue;
      const TV d = TV(Vc * m.Dhb[J * m.nInst + K]);
      const TV* xk = x + 5 * ((size_t)K * m.Nc + cl);
#pragma unroll
      for (int k = 0; k < 5; ++k) acc[k] += d * xk[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) y[5 * c + k] = acc[k];
}

// Cyclic couplings (the interface part of Amul, blockFvMatrix.C:386-407):
// y_c += sum over the cyclic faces of c of B_f x_partner, B_f holding the
// partner's rotation; one thread per row that owns cyclic faces, after k_spmv.
template <typename TB, typename TV>
__global__ void __launch_bounds__(128) k_cyc_mv(DevMesh m, const TB* __restrict__ cblk, const TV* __restrict__ x,
                                                TV* __restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m.ncrow) return;
  const int c = m.cyc_row[r];
  TV acc[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) acc[k] = y[5 * c + k];
  for (int e = m.cyc_ptr[r]; e < m.cyc_ptr[r + 1]; ++e) {
    const int pc = m.bpartner[m.cyc_face[e]];
    const TB* Bk = cblk + (size_t)e * 25;
    TV xj[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xj[k] = x[5 * pc + k];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      TV a = TV(0);
#pragma unroll
      for (int j = 0; j < 5; ++j) a += TV(Bk[5 * i + j]) * xj[j];
      acc[i] += a;
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) y[5 * c + k] = acc[k];
}

// ------------------------------------- fused A x + LU-SGS (two-level schedule)
// On a schedule of two levels where the first holds the rows without lower
// neighbours and the second the rows without upper neighbours (the
// colour-blocked numbering of a bipartite mesh), z = M^-1 A x takes three
// passes instead of SpMV + two sweeps, and the second-level rows read their
// (lower) blocks once for both the product and the forward sweep:
//   pass 1 (level-0 rows): w = (A x)_c
//   pass 2 (level-1 rows): y = (A x)_c; r' = y - sum_lower L (rD w)_j;
//                          w_c = rD_c r'   (forward + fused first reverse)
//   pass 3 (level-0 rows): the reverse sweep, as k_lusgs_level MODE 1.
// Same arithmetic as the separate kernels up to the order of the sums.
// SCALED: x is the unnormalised Krylov vector; the kernels use x * (1/beta)
// (the next basis vector) and store it in vout for their own rows, which
// removes the separate normalisation pass.  One reciprocal per thread: a
// division per gathered element would make the FP64 path ALU-bound.
template <bool SCALED, typename TV>
__device__ __forceinline__ TV ldx(const TV* __restrict__ x, size_t i, TV rbeta) {
  return SCALED ? x[i] * rbeta : x[i];
}
template <typename TV>
__device__ __forceinline__ TV krylov_rbeta(const KrylovScalars* ks) {
  return ks && ks->status == 0 ? TV(1.0 / ks->beta) : TV(1);
}
// the reciprocal norm of row c's system: its stacked case's, else the handle's
template <typename TV>
__device__ __forceinline__ TV row_rbeta(const DevMesh& m, int c, const KrylovScalars* ks) {
  if (m.caseBeta) {
    const int k = m.caseOf[c];
    return m.caseActive[k] && m.caseStatus[k] == 0 ? TV(1.0 / m.caseBeta[k]) : TV(1);
  }
  return krylov_rbeta<TV>(ks);
}

template <typename TB, typename TV, int MINB = 1, int UNR = 1, bool SCALED = false>
__global__ void __launch_bounds__(128, MINB) k_op_level0(DevMesh m, const TB* __restrict__ blk, const TB* __restrict__ dg,
                                                   const TV* __restrict__ x, TV* __restrict__ w,
                                                   const int* __restrict__ cells, int start, int count,
                                                   const KrylovScalars* __restrict__ ks, TV* __restrict__ vout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int c = cells ? cells[start + i] : start + i;
  const int s = c >> 5, lane = c & 31;
  const TV beta = SCALED ? row_rbeta<TV>(m, c, ks) : TV(1);  // reciprocal
  TV xc[5], acc[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) xc[k] = ldx<SCALED>(x, 5 * (size_t)c + k, beta);
  if (SCALED)
#pragma unroll
    for (int k = 0; k < 5; ++k) vout[5 * c + k] = xc[k];
  const TB* D = dg + (size_t)s * 25 * 32 + lane;
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    TV a = TV(0);
#pragma unroll
    for (int j = 0; j < 5; ++j) a += TV(D[(5 * r + j) * 32]) * xc[j];
    acc[r] = a;
  }
  const int base = m.slot_base[s];
  const int ns = m.nslot[c];
  const TV g = TV(m.gamma);
  // software pipeline over the slots: the column of slot t+2 and the
  // gathered x of slot t+1 are in flight while slot t is applied
  const int* __restrict__ sc = m.scol + (size_t)base * 32 + lane;
  int colA = ns > 0 ? sc[0] : 0;
  int colB = ns > 1 ? sc[32] : 0;
  TV xn[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) xn[k] = ns > 0 ? ldx<SCALED>(x, 5 * (size_t)colA + k, beta) : TV(0);
#pragma unroll UNR
  for (int t = 0; t < ns; ++t) {
    const int col = colA;
    TV xj[5], y[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xj[k] = xn[k];
    colA = colB;
    if (t + 2 < ns) colB = sc[(t + 2) * 32];
    if (t + 1 < ns)
#pragma unroll
      for (int k = 0; k < 5; ++k) xn[k] = ldx<SCALED>(x, 5 * (size_t)colA + k, beta);
    SlotBlock<TB> Bk;
    Bk.load(blk, base + t, lane);
    Bk.mv(g, xj, y);
    if (m.vjslot) vj_sub<TB>(m, base + t, lane, col, xj, y);
#pragma unroll
    for (int r = 0; r < 5; ++r) acc[r] += y[r];
  }
  if (m.nInst > 1 && hb_in_zone(m, c)) {
    const int J = c / m.Nc, cl = c - J * m.Nc;
    const double Vc = m.V[c];
    for (int K = 0; K < m.nInst; ++K) {
      if (K == J) continue;
      const TV d = TV(Vc * m.Dhb[J * m.nInst + K]);
      const TV* xk = x + 5 * ((size_t)K * m.Nc + cl);
#pragma unroll
      for (int k = 0; k < 5; ++k) acc[k] += d * ldx<SCALED>(xk, k, beta);
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) w[5 * c + k] = acc[k];
}

template <typename TB, typename TV, int MINB = 1, int UNR = 1, bool SCALED = false>
__global__ void __launch_bounds__(128, MINB) k_op_level1(DevMesh m, const TB* __restrict__ blk, const TB* __restrict__ dg,
                                                   const TB* __restrict__ rD, const TV* __restrict__ x,
                                                   TV* __restrict__ w, const int* __restrict__ cells, int start,
                                                   int count, const KrylovScalars* __restrict__ ks,
                                                   TV* __restrict__ vout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int c = cells ? cells[start + i] : start + i;
  const int s = c >> 5, lane = c & 31;
  const TV beta = SCALED ? row_rbeta<TV>(m, c, ks) : TV(1);  // reciprocal
  TV xc[5], acc[5], fw[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    xc[k] = ldx<SCALED>(x, 5 * (size_t)c + k, beta);
    fw[k] = TV(0);
  }
  if (SCALED)
#pragma unroll
    for (int k = 0; k < 5; ++k) vout[5 * c + k] = xc[k];
  const TB* D = dg + (size_t)s * 25 * 32 + lane;
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    TV a = TV(0);
#pragma unroll
    for (int j = 0; j < 5; ++j) a += TV(D[(5 * r + j) * 32]) * xc[j];
    acc[r] = a;
  }
  const int base = m.slot_base[s];
  const int ns = m.nslot[c];  // all lower: these rows have no upper neighbours
  const TV g = TV(m.gamma);
#pragma unroll UNR
  for (int t = 0; t < ns; ++t) {
    const int col = m.scol[(base + t) * 32 + lane];
    const TV rj = TV(rD[col]);
    TV xj[5], dj[5], ya[5], yb[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      xj[k] = ldx<SCALED>(x, 5 * (size_t)col + k, beta);
      dj[k] = rj * w[5 * col + k];
    }
    SlotBlock<TB> Bk;
    Bk.load(blk, base + t, lane);
    Bk.mv2(g, xj, ya, dj, yb);
    if (m.vjslot) {
      vj_sub<TB>(m, base + t, lane, col, xj, ya);
      vj_sub<TB>(m, base + t, lane, col, dj, yb);
    }
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      acc[r] += ya[r];
      fw[r] += yb[r];
    }
  }
  if (m.nInst > 1 && hb_in_zone(m, c)) {
    const int J = c / m.Nc, cl = c - J * m.Nc;
    const double Vc = m.V[c];
    for (int K = 0; K < m.nInst; ++K) {
      if (K == J) continue;
      const TV d = TV(Vc * m.Dhb[J * m.nInst + K]);
      const TV* xk = x + 5 * ((size_t)K * m.Nc + cl);
#pragma unroll
      for (int k = 0; k < 5; ++k) acc[k] += d * ldx<SCALED>(xk, k, beta);
    }
  }
  const TV rc = TV(rD[c]);
#pragma unroll
  for (int k = 0; k < 5; ++k) w[5 * c + k] = rc * (acc[k] - fw[k]);
}

// ------------------------------------------------------------------ LU-SGS
// SCALE: also apply the reverse step of a row without upper neighbours
// (delta = rD * r'), fusing the last forward level with the first reverse one.
template <typename TB, typename TV, bool SCALE = false>
__device__ __forceinline__ void lusgs_fwd_row(const DevMesh& m, const TB* __restrict__ blk, const TB* __restrict__ rD,
                                              TV* __restrict__ r, int c) {
  const int s = c >> 5, lane = c & 31;
  const int base = m.slot_base[s];
  const int nl = m.nlow[c];
  TV acc[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) acc[k] = r[5 * c + k];
  const TV g = TV(m.gamma);
#pragma unroll 1
  for (int t = 0; t < nl; ++t) {
    const int col = m.scol[(base + t) * 32 + lane];
    const TV rj = TV(rD[col]);
    TV dj[5], y[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) dj[k] = rj * r[5 * col + k];
    SlotBlock<TB> Bk;
    Bk.load(blk, base + t, lane);
    Bk.mv(g, dj, y);
    if (m.vjslot) vj_sub<TB>(m, base + t, lane, col, dj, y);
#pragma unroll
    for (int i = 0; i < 5; ++i) acc[i] -= y[i];
  }
  if (SCALE) {
    const TV rc = TV(rD[c]);
#pragma unroll
    for (int k = 0; k < 5; ++k) r[5 * c + k] = rc * acc[k];
  } else {
#pragma unroll
    for (int k = 0; k < 5; ++k) r[5 * c + k] = acc[k];
  }
}

template <typename TB, typename TV>
__device__ __forceinline__ void lusgs_rev_row(const DevMesh& m, const TB* __restrict__ blk, const TB* __restrict__ rD,
                                              TV* __restrict__ r, int c) {
  const int s = c >> 5, lane = c & 31;
  const int base = m.slot_base[s];
  const int nl = m.nlow[c], ns = m.nslot[c];
  TV acc[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) acc[k] = r[5 * c + k];
  // two slots in flight: their column loads and the dependent gathers overlap
  // (2% on the reverse sweep; a deeper software pipeline with the next slot's
  // column and deltas loaded ahead measured 11% slower)
  const TV g = TV(m.gamma);
#pragma unroll 2
  for (int t = ns - 1; t >= nl; --t) {
    const int col = m.scol[(base + t) * 32 + lane];
    TV dj[5], y[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) dj[k] = r[5 * col + k];
    SlotBlock<TB> Bk;
    Bk.load(blk, base + t, lane);
    Bk.mv(g, dj, y);
    if (m.vjslot) vj_sub<TB>(m, base + t, lane, col, dj, y);
#pragma unroll
    for (int i = 0; i < 5; ++i) acc[i] -= y[i];
  }
  const TV rc = TV(rD[c]);
#pragma unroll
  for (int k = 0; k < 5; ++k) r[5 * c + k] = rc * acc[k];
}

// Two rows of one reverse level in one thread: their slot loops run in
// lockstep, so the column index, block words and gathered neighbour rows of
// both are in flight together (a level's rows never read each other).  Each
// row's arithmetic is that of lusgs_rev_row: slots from the last down to the
// first upper one, acc -= B r_col, then the scaling by rD.
template <typename TB, typename TV>
__device__ __forceinline__ void lusgs_rev_row2(const DevMesh& m, const TB* __restrict__ blk,
                                               const TB* __restrict__ rD, TV* __restrict__ r, int c0, int c1) {
  const int l0 = c0 & 31, l1 = c1 & 31;
  const int b0 = m.slot_base[c0 >> 5], b1 = m.slot_base[c1 >> 5];
  const int nl0 = m.nlow[c0], nl1 = m.nlow[c1];
  int t0 = m.nslot[c0] - 1, t1 = m.nslot[c1] - 1;
  TV a0[5], a1[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    a0[k] = r[5 * c0 + k];
    a1[k] = r[5 * c1 + k];
  }
  const TV g = TV(m.gamma);
#pragma unroll 1
  for (; t0 >= nl0 || t1 >= nl1; --t0, --t1) {
    const bool v0 = t0 >= nl0, v1 = t1 >= nl1;
    const int col0 = v0 ? m.scol[(b0 + t0) * 32 + l0] : c0;
    const int col1 = v1 ? m.scol[(b1 + t1) * 32 + l1] : c1;
    TV d0[5], d1[5], y0[5], y1[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      d0[k] = r[5 * col0 + k];
      d1[k] = r[5 * col1 + k];
    }
    SlotBlock<TB> B0, B1;
    if (v0) B0.load(blk, b0 + t0, l0);
    if (v1) B1.load(blk, b1 + t1, l1);
    if (v0) {
      B0.mv(g, d0, y0);
      if (m.vjslot) vj_sub<TB>(m, b0 + t0, l0, col0, d0, y0);
#pragma unroll
      for (int i = 0; i < 5; ++i) a0[i] -= y0[i];
    }
    if (v1) {
      B1.mv(g, d1, y1);
      if (m.vjslot) vj_sub<TB>(m, b1 + t1, l1, col1, d1, y1);
#pragma unroll
      for (int i = 0; i < 5; ++i) a1[i] -= y1[i];
    }
  }
  const TV rc0 = TV(rD[c0]), rc1 = TV(rD[c1]);
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    r[5 * c0 + k] = rc0 * a0[k];
    r[5 * c1 + k] = rc1 * a1[k];
  }
}

// reverse level with two rows per thread: rows i and i + ceil(count/2)
template <typename TB, typename TV>
__global__ void __launch_bounds__(128) k_lusgs_rev2(DevMesh m, const TB* __restrict__ blk, const TB* __restrict__ rD,
                                                    TV* __restrict__ r, const int* __restrict__ cells, int start,
                                                    int count) {
  const int half = (count + 1) >> 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= half) return;
  const int c0 = cells ? cells[start + i] : start + i;
  if (i + half < count)
    lusgs_rev_row2<TB, TV>(m, blk, rD, r, c0, cells ? cells[start + i + half] : start + i + half);
  else
    lusgs_rev_row<TB, TV>(m, blk, rD, r, c0);
}

// one launch per level: cells = level list (nullptr when the level is the
// contiguous range [start, start+count))
// MODE 0: forward row, 1: reverse row, 2: forward row + reverse scaling
template <typename TB, typename TV, int MODE>
__global__ void __launch_bounds__(128) k_lusgs_level(DevMesh m, const TB* __restrict__ blk,
                                                     const TB* __restrict__ rD, TV* __restrict__ r,
                                                     const int* __restrict__ cells, int start, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int c = cells ? cells[start + i] : start + i;
  if (MODE == 0)
    lusgs_fwd_row<TB, TV>(m, blk, rD, r, c);
  else if (MODE == 1)
    lusgs_rev_row<TB, TV>(m, blk, rD, r, c);
  else
    lusgs_fwd_row<TB, TV, true>(m, blk, rD, r, c);
}

// one CTA walks every level (small meshes / many tiny levels)
template <typename TB, typename TV, bool FWD>
__global__ void __launch_bounds__(1024) k_lusgs_block(DevMesh m, const TB* __restrict__ blk,
                                                      const TB* __restrict__ rD, TV* __restrict__ r,
                                                      const int* __restrict__ cells, const int* __restrict__ lptr,
                                                      int nlev) {
  for (int l = 0; l < nlev; ++l) {
    const int a = lptr[l], b = lptr[l + 1];
    for (int i = a + threadIdx.x; i < b; i += blockDim.x) {
      const int c = cells[i];
      if (FWD)
        lusgs_fwd_row<TB, TV>(m, blk, rD, r, c);
      else
        lusgs_rev_row<TB, TV>(m, blk, rD, r, c);
    }
    __syncthreads();
  }
}

// ----------------------------------------------- sync-free LU-SGS sweeps
// One launch per sweep for schedules with many levels (RCM / natural
// numbering): blocks draw consecutive tickets in level order (order[]), so a
// row only ever waits for rows with smaller tickets, whose blocks started
// earlier and are resident or done -- no deadlock.  The sweep writes its rows
// into a padded output array (8 words per row, 32 B for FP32) that starts
// filled with a sentinel (all bits set: a NaN with the sign bit, which GPU
// arithmetic does not produce from finite operands -- a result that matched
// it, from a NaN already in the input, would make its dependents give up
// at the bound and report, never hang), and a row's result
// words are their own done flags: a row polls its neighbours' five words
// with relaxed loads until none is the sentinel.  One L2 round trip per
// poll brings both the readiness and the values, the writer needs no fence,
// and the polls of all prefetched neighbours are issued together.  The
// arithmetic per row is that of lusgs_fwd_row / lusgs_rev_row, so the result
// equals the level-by-level sweep bit for bit.  A wait that exceeds the
// bound sets status bit 8, publishes zeros (so that its dependents do not
// wait in turn) and returns; waiting rows that see bit 8 give up too (the
// host reports ICS_ERR_TIMEOUT).
constexpr int SWEEP_SPIN_LIMIT = 1 << 22;
constexpr int SWEEP_PAD = 8;  // words per row of the sweep outputs
// rows per block: a level's rows are consecutive tickets, so small blocks
// spread each level over more SMs (FP64 sweeps 4% faster than with 128-row
// blocks on a 285-level RCM box; FP32 unchanged)
constexpr int SWEEP_THREADS = 32;

__device__ __forceinline__ int ld_relaxed_int(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void ld_relaxed5(const float* p, float* v) {
  asm volatile("ld.relaxed.gpu.global.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
               : "l"(p)
               : "memory");
  asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v[4]) : "l"(p + 4) : "memory");
}
__device__ __forceinline__ void ld_relaxed5(const double* p, double* v) {
  asm volatile("ld.relaxed.gpu.global.v2.f64 {%0, %1}, [%2];" : "=d"(v[0]), "=d"(v[1]) : "l"(p) : "memory");
  asm volatile("ld.relaxed.gpu.global.v2.f64 {%0, %1}, [%2];" : "=d"(v[2]), "=d"(v[3]) : "l"(p + 2) : "memory");
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v[4]) : "l"(p + 4) : "memory");
}
__device__ __forceinline__ void st_relaxed5(float* p, const float* v) {
  asm volatile("st.relaxed.gpu.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v[0]), "f"(v[1]), "f"(v[2]),
               "f"(v[3])
               : "memory");
  asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p + 4), "f"(v[4]) : "memory");
}
__device__ __forceinline__ void st_relaxed5(double* p, const double* v) {
  asm volatile("st.relaxed.gpu.global.v2.f64 [%0], {%1, %2};" ::"l"(p), "d"(v[0]), "d"(v[1]) : "memory");
  asm volatile("st.relaxed.gpu.global.v2.f64 [%0], {%1, %2};" ::"l"(p + 2), "d"(v[2]), "d"(v[3]) : "memory");
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p + 4), "d"(v[4]) : "memory");
}
__device__ __forceinline__ bool sweep_word_set(float v) { return __float_as_uint(v) != 0xffffffffu; }
__device__ __forceinline__ bool sweep_word_set(double v) {
  return (unsigned long long)__double_as_longlong(v) != ~0ull;
}
template <typename TV>
__device__ __forceinline__ bool sweep_ready(const TV* v) {
  return sweep_word_set(v[0]) && sweep_word_set(v[1]) && sweep_word_set(v[2]) && sweep_word_set(v[3]) &&
         sweep_word_set(v[4]);
}

// FWD: in = the right-hand side r (5 words per row), out = the forward
// result; !FWD: in = the forward result (padded), out = the reverse result,
// also written to r (5 words per row).  `out` holds the sentinel on entry.
template <typename TB, typename TV, bool FWD>
__global__ void __launch_bounds__(SWEEP_THREADS) k_lusgs_sweep(DevMesh m, const TB* __restrict__ blk,
                                                     const TB* __restrict__ rD, const TV* in, TV* out, TV* r,
                                                     const int* __restrict__ order, int count, unsigned int* ticket,
                                                     int* status, int spin_limit) {
  __shared__ int base;
  if (threadIdx.x == 0) base = (int)atomicAdd(ticket, blockDim.x);
  __syncthreads();
  const int i = base + threadIdx.x;
  if (i >= count) return;
  const int c = order[i];
  const int s = c >> 5, lane = c & 31;
  const int sb = m.slot_base[s];
  const int nl = m.nlow[c], ns = m.nslot[c];
  // the neighbours of this sweep: slots [0, nl) forward, [nl, ns) backward
  const int nn = FWD ? nl : ns - nl;
  auto slot = [&](int p) { return FWD ? p : ns - 1 - p; };
  // everything that does not depend on the neighbours' results (columns,
  // blocks, their rD) is loaded before the first poll
  constexpr int PF = 3;
  int colp[PF];
  SlotBlock<TB> bp[PF];
  TV rdp[PF];
#pragma unroll
  for (int p = 0; p < PF; ++p) {
    if (p < nn) {
      const int t = slot(p);
      colp[p] = m.scol[(sb + t) * 32 + lane];
      bp[p].load(blk, sb + t, lane);
      rdp[p] = FWD ? TV(rD[colp[p]]) : TV(1);
    }
  }
  const TV g = TV(m.gamma);
  TV acc[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) acc[k] = FWD ? __ldcg(in + 5 * c + k) : __ldcg(in + SWEEP_PAD * c + k);
  TV* mine = out + (size_t)SWEEP_PAD * c;
  // poll the prefetched neighbours together: (bounded; gives up on bit 8)
  TV rv[PF][5];
  unsigned pending = 0;
#pragma unroll
  for (int p = 0; p < PF; ++p)
    if (p < nn) pending |= 1u << p;
  {
    int it = 0;
    unsigned ns_ = 32;
    while (true) {
#pragma unroll
      for (int p = 0; p < PF; ++p)
        if (pending & (1u << p)) {
          ld_relaxed5(out + (size_t)SWEEP_PAD * colp[p], rv[p]);
          if (sweep_ready(rv[p])) pending &= ~(1u << p);
        }
      if (!pending) break;
      ++it;
      if (it > spin_limit || ((it & 63) == 0 && (ld_relaxed_int(status) & 8))) {
        if (it > spin_limit) atomicOr(status, 8);
        const TV z[5] = {TV(0), TV(0), TV(0), TV(0), TV(0)};
        st_relaxed5(mine, z);
        return;
      }
      __nanosleep(ns_);
      if (ns_ < 256) ns_ <<= 1;
    }
  }
#pragma unroll
  for (int p = 0; p < PF; ++p) {
    if (p < nn) {
      TV dj[5], y[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) dj[k] = rdp[p] * rv[p][k];
      bp[p].mv(g, dj, y);
      if (m.vjslot) vj_sub<TB>(m, sb + slot(p), lane, colp[p], dj, y);
#pragma unroll
      for (int a = 0; a < 5; ++a) acc[a] -= y[a];
    }
  }
#pragma unroll 1
  for (int p = PF; p < nn; ++p) {  // rows with more neighbours than prefetched
    const int t = slot(p);
    const int col = m.scol[(sb + t) * 32 + lane];
    TV rj5[5];
    int it = 0;
    unsigned ns_ = 32;
    while (true) {
      ld_relaxed5(out + (size_t)SWEEP_PAD * col, rj5);
      if (sweep_ready(rj5)) break;
      ++it;
      if (it > spin_limit || ((it & 63) == 0 && (ld_relaxed_int(status) & 8))) {
        if (it > spin_limit) atomicOr(status, 8);
        const TV z[5] = {TV(0), TV(0), TV(0), TV(0), TV(0)};
        st_relaxed5(mine, z);
        return;
      }
      __nanosleep(ns_);
      if (ns_ < 256) ns_ <<= 1;
    }
    const TV rj = FWD ? TV(rD[col]) : TV(1);
    TV dj[5], y[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) dj[k] = rj * rj5[k];
    SlotBlock<TB> Bk;
    Bk.load(blk, sb + t, lane);
    Bk.mv(g, dj, y);
    if (m.vjslot) vj_sub<TB>(m, sb + t, lane, col, dj, y);
#pragma unroll
    for (int a = 0; a < 5; ++a) acc[a] -= y[a];
  }
  if (!FWD) {
    const TV rc = TV(rD[c]);
#pragma unroll
    for (int k = 0; k < 5; ++k) acc[k] = rc * acc[k];
#pragma unroll
    for (int k = 0; k < 5; ++k) r[5 * c + k] = acc[k];
  }
  st_relaxed5(mine, acc);
}

template <typename TB, typename TV>
__global__ void k_jacobi_apply(int N, const TB* __restrict__ inv, TV* __restrict__ r) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const int s = c >> 5, lane = c & 31;
  const TB* D = inv + (size_t)s * 25 * 32 + lane;
  TV x[5], z[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) x[k] = r[5 * c + k];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    TV a = TV(0);
#pragma unroll
    for (int j = 0; j < 5; ++j) a += TV(D[(5 * i + j) * 32]) * x[j];
    z[i] = a;
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) r[5 * c + k] = z[k];
}

// ------------------------------------------------------------ vector kernels
template <typename TS, typename TD>
__global__ void k_cast(long n, const TS* __restrict__ a, TD* __restrict__ b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = TD(a[i]);
}

// start of a cycle: beta = sqrt(sum), bh = (beta, 0...)
__device__ __forceinline__ void dev_beta0(KrylovScalars* ks, int m) {
  const double beta = sqrt(ks->red[0]);
  ks->beta = beta;
  for (int i = 0; i <= m; ++i) ks->bh[i] = 0.0;
  ks->bh[0] = beta;
  if (!(beta > 0.0)) ks->status = isfinite(beta) ? 2 : 4;
}

__device__ __forceinline__ void givens(double h, double beta, double& c, double& s) {
  if (beta == 0) {
    c = 1;
    s = 0;
  } else if (fabs(beta) > fabs(h)) {
    const double tau = -h / beta;
    s = 1.0 / sqrt(1.0 + tau * tau);
    c = s * tau;
  } else {
    const double tau = -beta / h;
    c = 1.0 / sqrt(1.0 + tau * tau);
    s = c * tau;
  }
}

// after MGS of direction i: H[j][i] for j <= i are in H, red[1] holds |w|^2;
// rotate column i with the previous Givens rotations and make a new one
// (gmres.C:1013-1027, rotation gmres.C:44-69)
__device__ __forceinline__ void dev_hess(KrylovScalars* ks, int i, int m) {
  if (ks->status) return;
  double* H = ks->H;
  const double beta = sqrt(ks->red[1]);
  for (int j = 0; j < i; ++j) {
    const double Hji = H[j * m + i];
    H[j * m + i] = ks->c[j] * Hji - ks->s[j] * H[(j + 1) * m + i];
    H[(j + 1) * m + i] = ks->s[j] * Hji + ks->c[j] * H[(j + 1) * m + i];
  }
  givens(H[i * m + i], beta, ks->c[i], ks->s[i]);
  const double bhi = ks->bh[i];
  ks->bh[i] = ks->c[i] * bhi - ks->s[i] * ks->bh[i + 1];
  ks->bh[i + 1] = ks->s[i] * bhi + ks->c[i] * ks->bh[i + 1];
  H[i * m + i] = ks->c[i] * H[i * m + i] - ks->s[i] * beta;
  ks->beta = beta;
}

// w -= hprev * vprev (when vprev), then sum w.vnext (or w.w) -> out.
// post = 1: the finishing thread also starts the cycle (dev_beta0);
// post = 2: it also performs the Hessenberg update of direction i.
template <typename TV>
__global__ void __launch_bounds__(RB, 4) k_mgs(long n, TV* __restrict__ w, const TV* __restrict__ vprev,
                                            const double* __restrict__ hprev, const TV* __restrict__ vnext,
                                            const int* __restrict__ status, double* __restrict__ partials,
                                            unsigned int* __restrict__ counter, double* __restrict__ out,
                                            KrylovScalars* __restrict__ ks, int post, int dir, int m) {
  double acc[1] = {0.0};
  if (*status == 0) {
    const TV h = vprev ? TV(*hprev) : TV(0);
    using VT = typename V16<TV>::T;
    constexpr int L = V16<TV>::n;
    const long nv = n / L;  // 16-byte chunks (vectors start 256-byte aligned)
    VT* w4 = reinterpret_cast<VT*>(w);
    const VT* p4 = reinterpret_cast<const VT*>(vprev);
    const VT* o4 = reinterpret_cast<const VT*>(vnext);
    const long stride = (long)gridDim.x * blockDim.x;
    TV tacc = TV(0);
    // MGS_CHUNKS 16-byte chunks per thread and iteration, every load issued
    // before the first use: the compiler's unrolled loop kept one chunk in
    // flight at 32 registers (ncu: long-scoreboard stalls, 50% warps active);
    // two chunks at <= 64 registers measured 6% faster per step
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    for (; i + (MGS_CHUNKS - 1) * stride < nv; i += MGS_CHUNKS * stride) {
      VT x[MGS_CHUNKS], pv[MGS_CHUNKS], ov[MGS_CHUNKS];
#pragma unroll
      for (int u = 0; u < MGS_CHUNKS; ++u) {
        x[u] = w4[i + u * stride];
        if (vprev) pv[u] = p4[i + u * stride];
        if (vnext) ov[u] = o4[i + u * stride];
      }
#pragma unroll
      for (int u = 0; u < MGS_CHUNKS; ++u) {
        if (vprev) {
          axpy16(x[u], h, pv[u]);
          w4[i + u * stride] = x[u];
        }
        tacc += dot16(x[u], vnext ? ov[u] : x[u]);
      }
    }
    for (; i < nv; i += stride) {
      VT x = w4[i];
      if (vprev) {
        axpy16(x, h, p4[i]);
        w4[i] = x;
      }
      tacc += dot16(x, vnext ? o4[i] : x);
    }
    for (long i = nv * L + blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride) {
      TV x = w[i];
      if (vprev) {
        x = x - h * vprev[i];
        w[i] = x;
      }
      const TV o = vnext ? vnext[i] : x;
      tacc += x * o;
    }
    acc[0] = double(tacc);
  }
  if (reduce_finish<1>(acc, partials, counter, out)) {
    if (post == 1)
      dev_beta0(ks, m);
    else if (post == 2)
      dev_hess(ks, dir, m);
  }
}

__device__ __forceinline__ float4 div16(float4 x, float b) { return make_float4(x.x / b, x.y / b, x.z / b, x.w / b); }
__device__ __forceinline__ double2 div16(double2 x, double b) { return make_double2(x.x / b, x.y / b); }
__device__ __forceinline__ void addmul16(float4& a, float y, const float4& v) {
  a.x += y * v.x;
  a.y += y * v.y;
  a.z += y * v.z;
  a.w += y * v.w;
}
__device__ __forceinline__ void addmul16(double2& a, double y, const double2& v) {
  a.x += y * v.x;
  a.y += y * v.y;
}

// v = w / beta (gmres.C: sV = sTmp/beta)
template <typename TV>
__global__ void k_scale(long n, const TV* __restrict__ w, TV* __restrict__ v, const KrylovScalars* __restrict__ ks) {
  if (ks->status) return;
  const TV beta = TV(ks->beta);
  using VT = typename V16<TV>::T;
  constexpr int L = V16<TV>::n;
  const long nv = n / L;
  const long stride = (long)gridDim.x * blockDim.x;
  const VT* w4 = reinterpret_cast<const VT*>(w);
  VT* v4 = reinterpret_cast<VT*>(v);
#pragma unroll 4
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nv; i += stride) v4[i] = div16(w4[i], beta);
  for (long i = nv * L + blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride) v[i] = w[i] / beta;
}

__global__ void k_backsub(KrylovScalars* ks, int m) {
  if (ks->status) return;
  for (int i = m - 1; i >= 0; --i) {
    double sum = ks->bh[i];
    for (int j = i + 1; j < m; ++j) sum -= ks->H[i * m + j] * ks->y[j];
    const double hii = ks->H[i * m + i];
    const double st = hii >= 0 ? hii + VSMALL : hii - VSMALL;
    ks->y[i] = sum / st;
  }
}

template <typename TV>
__global__ void k_xupdate(long n, TV* __restrict__ x, const TV* __restrict__ V, const KrylovScalars* __restrict__ ks,
                          int m, long vstride) {
  if (ks->status) return;
  using VT = typename V16<TV>::T;
  constexpr int L = V16<TV>::n;
  const long nv = n / L;
  const long stride = (long)gridDim.x * blockDim.x;
  VT* x4 = reinterpret_cast<VT*>(x);
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nv; q += stride) {
    VT a = x4[q];
    for (int i = 0; i < m; ++i)
      addmul16(a, TV(ks->y[i]), reinterpret_cast<const VT*>(V + (size_t)i * vstride)[q]);
    x4[q] = a;
  }
  for (long q = nv * L + blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += stride) {
    TV a = x[q];
    for (int i = 0; i < m; ++i) a += TV(ks->y[i]) * V[(size_t)i * vstride + q];
    x[q] = a;
  }
}

// Per-instance reductions: blockIdx.y is the instance, whose Nc cells start at
// y*Nc; each instance folds its own partials and counter into out + y*NV.
#define ICS_INSTANCE_RANGE(Nc)                                     \
  const int inst_ = blockIdx.y;                                    \
  const int cend_ = (inst_ + 1) * (Nc);                            \
  partials += (size_t)inst_ * gridDim.x * NV_;                     \
  counter += inst_;                                                \
  out += inst_ * NV_;

// r = b - t, per-equation L1 sums of r (rho, rhoUx, rhoUy, rhoUz, rhoE)
template <typename TV>
__global__ void __launch_bounds__(RB) k_resid(int Nc, const double* __restrict__ b, const TV* __restrict__ t,
                                              TV* __restrict__ r, double* __restrict__ partials,
                                              unsigned int* __restrict__ counter, double* __restrict__ out) {
  constexpr int NV_ = 5;
  ICS_INSTANCE_RANGE(Nc)
  double acc[5] = {0, 0, 0, 0, 0};
  for (int c = inst_ * Nc + blockIdx.x * blockDim.x + threadIdx.x; c < cend_; c += gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const TV v = TV(b[5 * c + k]) - t[5 * c + k];
      r[5 * c + k] = v;
      acc[k] += fabs(double(v));
    }
  }
  reduce_finish<5>(acc, partials, counter, out);
}

// sums of |b_k| (initial residual) and the norm factors
template <typename TV>
__global__ void __launch_bounds__(RB) k_normfac(int Nc, const double* __restrict__ b, const TV* __restrict__ t,
                                                double* __restrict__ partials, unsigned int* __restrict__ counter,
                                                double* __restrict__ out) {
  // out per instance: nf_rho, nf_rhoE, nf_rhoU, |b| rho, Ux, Uy, Uz, rhoE
  constexpr int NV_ = 8;
  ICS_INSTANCE_RANGE(Nc)
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int c = inst_ * Nc + blockIdx.x * blockDim.x + threadIdx.x; c < cend_; c += gridDim.x * blockDim.x) {
    const double t0 = double(t[5 * c]), t4 = double(t[5 * c + 4]);
    const double t1 = double(t[5 * c + 1]), t2 = double(t[5 * c + 2]), t3 = double(t[5 * c + 3]);
    const double b0 = b[5 * c], b1 = b[5 * c + 1], b2 = b[5 * c + 2], b3 = b[5 * c + 3], b4 = b[5 * c + 4];
    acc[0] += fabs(t0) + fabs(b0);
    acc[1] += fabs(t4) + fabs(b4);
    acc[2] += sqrt(t1 * t1 + t2 * t2 + t3 * t3) + sqrt(b1 * b1 + b2 * b2 + b3 * b3);
    acc[3] += fabs(b0);
    acc[4] += fabs(b1);
    acc[5] += fabs(b2);
    acc[6] += fabs(b3);
    acc[7] += fabs(b4);
  }
  reduce_finish<8>(acc, partials, counter, out);
}

__global__ void __launch_bounds__(RB) k_wsum(int Nc, const double* __restrict__ W, double* __restrict__ partials,
                                             unsigned int* __restrict__ counter, double* __restrict__ out) {
  constexpr int NV_ = 5;
  ICS_INSTANCE_RANGE(Nc)
  double acc[5] = {0, 0, 0, 0, 0};
  for (int c = inst_ * Nc + blockIdx.x * blockDim.x + threadIdx.x; c < cend_; c += gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < 5; ++k) acc[k] += W[5 * c + k];
  reduce_finish<5>(acc, partials, counter, out);
}

template <typename TV>
__global__ void k_wmavg(int N, int Nc, const double* __restrict__ W, const KrylovScalars* __restrict__ ks,
                        TV* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const double* avg = ks->avg + 5 * (c / Nc);
#pragma unroll
  for (int k = 0; k < 5; ++k) out[5 * c + k] = TV(W[5 * c + k] - avg[k]);
}

// instance averages (gAverage per field) from the instance sums
__global__ void k_avg(KrylovScalars* ks, int Nc, int nInst) {
  for (int k = 0; k < 5 * nInst; ++k) ks->avg[k] = ks->avg[k] / Nc;
}

template <typename TV>
__global__ void k_to_dW(int N, const TV* __restrict__ x, double* __restrict__ dW, int s0, int s1, int s2) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  dW[5 * c] = double(x[5 * c]);
  dW[5 * c + 1] = s0 == -1 ? 0.0 : double(x[5 * c + 1]);
  dW[5 * c + 2] = s1 == -1 ? 0.0 : double(x[5 * c + 2]);
  dW[5 * c + 3] = s2 == -1 ? 0.0 : double(x[5 * c + 3]);
  dW[5 * c + 4] = double(x[5 * c + 4]);
}

__global__ void __launch_bounds__(RB) k_sumsq(int N, const double* __restrict__ a, double* __restrict__ partials,
                                              unsigned int* __restrict__ counter, double* __restrict__ out) {
  double acc[1] = {0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) acc[0] += a[c];
  reduce_finish<1>(acc, partials, counter, out);
}

// -------------------------------------------------------------- dispatch
template <typename TB, typename TV>
static void spmv_t(Handle& h, const TV* x, TV* y) {
  ICS_LAUNCH(h, ICS_K_SPMV, k_spmv<TB, TV><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m, (const TB*)h.blk, (const TB*)h.dg, x, y));
  if (h.m.ncrow > 0)
    ICS_LAUNCH(h, ICS_K_SPMV, k_cyc_mv<TB, TV><<<grid_for(h.m.ncrow, 128), 128, 0, h.stream>>>(h.m, (const TB*)h.cblk, x, y));
}


// one reverse level: one row per thread, or two (Handle::tuneRevRows)
template <typename TB, typename TV>
static void rev_level(Handle& h, const TB* blk, const TB* rD, TV* r, const int* cells, int start, int cnt) {
  if (h.tuneRevRows == 2)
    ICS_LAUNCH(h, ICS_K_LUSGS_REV, k_lusgs_rev2<TB, TV><<<grid_for((cnt + 1) / 2, 128), 128, 0, h.stream>>>(
                                       h.m, blk, rD, r, cells, start, cnt));
  else
    ICS_LAUNCH(h, ICS_K_LUSGS_REV, k_lusgs_level<TB, TV, 1><<<grid_for(cnt, 128), 128, 0, h.stream>>>(
                                       h.m, blk, rD, r, cells, start, cnt));
}

template <typename TB, typename TV>
static void lusgs_t(Handle& h, TV* r, const TB* blkIn = nullptr, const TB* rDIn = nullptr) {
  const DevMesh& m = h.m;
  const TB* blk = blkIn ? blkIn : (const TB*)h.blk;
  const TB* rD = rDIn ? rDIn : (const TB*)h.rD;
  // forward sweep, then reverse sweep; many small levels run in one CTA
  if ((long)m.N < 2048L * m.nfl) {
    ICS_LAUNCH(h, ICS_K_LUSGS_FWD, k_lusgs_block<TB, TV, true><<<1, 1024, 0, h.stream>>>(m, blk, rD, r, m.fl_cells, m.fl_lptr, m.nfl));
    if ((long)m.N < 2048L * m.nrl) {
      ICS_LAUNCH(h, ICS_K_LUSGS_REV,
                 k_lusgs_block<TB, TV, false><<<1, 1024, 0, h.stream>>>(m, blk, rD, r, m.rl_cells, m.rl_lptr, m.nrl));
      return;
    }
  }
  // Level launches.  Forward level 0 has no lower neighbours (r' = r): skipped.
  // When the last forward level holds exactly the rows of the first reverse
  // level (rows without upper neighbours, e.g. the last colour), the two are
  // fused: r' = r - L d*, then delta = rD r' in the same pass.
  // many levels on a large mesh: one sync-free launch per sweep
  if (m.nfl > 2 && (long)m.N >= 2048L * m.nfl) {
    cudaStream_t st = h.stream;
    int* status = &h.ks->status;
    TV* fwd = (TV*)m.sweep_pad;
    TV* rev = fwd + (size_t)SWEEP_PAD * m.N;
    const size_t padBytes = (size_t)SWEEP_PAD * m.N * sizeof(TV);
    ICS_CUDA(cudaMemsetAsync(fwd, 0xff, 2 * padBytes, st));  // the sentinel in both outputs
    ICS_CUDA(cudaMemsetAsync(m.sweep_ticket, 0, 2 * sizeof(unsigned int), st));
    ICS_LAUNCH(h, ICS_K_LUSGS_FWD, k_lusgs_sweep<TB, TV, true><<<grid_for(m.N, SWEEP_THREADS), SWEEP_THREADS, 0, st>>>(
                                       m, blk, rD, r, fwd, nullptr, m.fl_cells, m.N, m.sweep_ticket, status,
                                       SWEEP_SPIN_LIMIT));
    ICS_LAUNCH(h, ICS_K_LUSGS_REV, k_lusgs_sweep<TB, TV, false><<<grid_for(m.N, SWEEP_THREADS), SWEEP_THREADS, 0, st>>>(
                                       m, blk, rD, fwd, rev, r, m.rl_cells, m.N, m.sweep_ticket + 1, status,
                                       SWEEP_SPIN_LIMIT));
    return;
  }
  const bool blockFwd = (long)m.N < 2048L * m.nfl;
  const bool fuse = !blockFwd && m.fuse_last;
  if (!blockFwd) {
    for (int l = 0; l < m.nfl; ++l) {
      const bool last = l == m.nfl - 1;
      if (l == 0 && !(fuse && last)) continue;
      const int a = m.fl_ptr[l], cnt = m.fl_ptr[l + 1] - a;
      const bool contig = m.fl_cstart[l] >= 0;
      const int* cells = contig ? nullptr : m.fl_cells;
      const int start = contig ? m.fl_cstart[l] : a;
      if (fuse && last)
        ICS_LAUNCH(h, ICS_K_LUSGS_FWD, k_lusgs_level<TB, TV, 2><<<grid_for(cnt, 128), 128, 0, h.stream>>>(
                                           m, blk, rD, r, cells, start, cnt));
      else
        ICS_LAUNCH(h, ICS_K_LUSGS_FWD, k_lusgs_level<TB, TV, 0><<<grid_for(cnt, 128), 128, 0, h.stream>>>(
                                           m, blk, rD, r, cells, start, cnt));
    }
  }
  if ((long)m.N < 2048L * m.nrl) {
    ICS_LAUNCH(h, ICS_K_LUSGS_REV,
               k_lusgs_block<TB, TV, false><<<1, 1024, 0, h.stream>>>(m, blk, rD, r, m.rl_cells, m.rl_lptr, m.nrl));
  } else {
    for (int l = fuse ? 1 : 0; l < m.nrl; ++l) {
      const int a = m.rl_ptr[l], cnt = m.rl_ptr[l + 1] - a;
      const bool contig = m.rl_cstart[l] >= 0;
      rev_level<TB, TV>(h, blk, rD, r, contig ? nullptr : m.rl_cells, contig ? m.rl_cstart[l] : a, cnt);
    }
  }
}

// w = M^-1 A x with M the LU-SGS preconditioner; true when the fused
// three-pass form applies (two levels, the second without upper neighbours,
// level launches rather than the single-CTA walk)
template <typename TB, typename TV>
static bool fused_op_available(const Handle& h) {
  const DevMesh& m = h.m;
  // (the fused passes carry no cyclic couplings: those meshes take spmv_t)
  return h.tuneFused && h.cfg.c.preconditioner == ICS_PC_LUSGS && m.nfl == 2 && m.nrl == 2 && m.fuse_last &&
         (long)m.N >= 2048L * m.nfl && m.ncyc == 0;
}

// vout != nullptr: x is unnormalised; v = x / beta is stored in vout and
// w = M^-1 A v (w must then differ from x)
template <typename TB, typename TV>
static bool fused_op_t(Handle& h, const TV* x, TV* w, TV* vout = nullptr) {
  const DevMesh& m = h.m;
  if (!fused_op_available<TB, TV>(h)) return false;
  const TB* blk = (const TB*)h.blk;
  const TB* dg = (const TB*)h.dg;
  const TB* rD = (const TB*)h.rD;
  auto level = [&](int l, const int** cells, int* start, int* cnt) {
    const int a = m.fl_ptr[l];
    *cnt = m.fl_ptr[l + 1] - a;
    const bool contig = m.fl_cstart[l] >= 0;
    *cells = contig ? nullptr : m.fl_cells;
    *start = contig ? m.fl_cstart[l] : a;
  };
  const int* c0;
  const int* c1;
  int s0, n0, s1, n1;
  level(0, &c0, &s0, &n0);
  level(1, &c1, &s1, &n1);
  // slot loops not unrolled; FP32: at least 8 blocks of 128 per SM (64
  // registers), with the factored slots 4-7% faster per pass than two slots
  // in flight or the compiler's register choice (72-80), and 10 or 12 blocks
  // (51 / 40 registers, the latter spilling) were not faster; FP64 would spill
  constexpr int OPB = sizeof(TB) == 4 ? 8 : 1;
  const KrylovScalars* ks = h.ks;
  if (n0) {
    if (vout)
      ICS_LAUNCH(h, ICS_K_OP0, k_op_level0<TB, TV, OPB, 1, true><<<grid_for(n0, 128), 128, 0, h.stream>>>(
                                   m, blk, dg, x, w, c0, s0, n0, ks, vout));
    else
      ICS_LAUNCH(h, ICS_K_OP0, k_op_level0<TB, TV, OPB, 1><<<grid_for(n0, 128), 128, 0, h.stream>>>(
                                   m, blk, dg, x, w, c0, s0, n0, nullptr, nullptr));
  }
  if (n1) {
    if (vout)
      ICS_LAUNCH(h, ICS_K_OP1, k_op_level1<TB, TV, OPB, 1, true><<<grid_for(n1, 128), 128, 0, h.stream>>>(
                                   m, blk, dg, rD, x, w, c1, s1, n1, ks, vout));
    else
      ICS_LAUNCH(h, ICS_K_OP1, k_op_level1<TB, TV, OPB, 1><<<grid_for(n1, 128), 128, 0, h.stream>>>(
                                   m, blk, dg, rD, x, w, c1, s1, n1, nullptr, nullptr));
  }
  // reverse level 1 = forward level 0 rows
  const int a = m.rl_ptr[1], cnt = m.rl_ptr[2] - a;
  const bool contig = m.rl_cstart[1] >= 0;
  if (cnt) rev_level<TB, TV>(h, blk, rD, w, contig ? nullptr : m.rl_cells, contig ? m.rl_cstart[1] : a, cnt);
  return true;
}

template <typename TB, typename TV>
static void precondition_t(Handle& h, TV* r) {
  if (h.cfg.c.preconditioner == ICS_PC_LUSGS)
    lusgs_t<TB, TV>(h, r);
  else if (h.cfg.c.preconditioner == ICS_PC_JACOBI)
    ICS_LAUNCH(h, ICS_K_JACOBI, k_jacobi_apply<TB, TV><<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m.N, (const TB*)h.dginv, r));
}

// One sync-free forward sweep over `order` (count rows) with a given wait
// bound; used to exercise the bounded waits (a row left out of the order
// never writes its result, so its dependents must give up and report).
template <typename TB, typename TV>
static void sweep_probe_t(Handle& h, const int* order, int count, int spin_limit) {
  const DevMesh& m = h.m;
  cudaStream_t st = h.stream;
  TV* fwd = (TV*)m.sweep_pad;
  ICS_CUDA(cudaMemsetAsync(fwd, 0xff, (size_t)SWEEP_PAD * m.N * sizeof(TV), st));
  ICS_CUDA(cudaMemsetAsync(m.sweep_ticket, 0, 2 * sizeof(unsigned int), st));
  ICS_CUDA(cudaMemsetAsync(h.kw, 0, 5ull * m.N * sizeof(TV), st));
  ICS_LAUNCH(h, ICS_K_LUSGS_FWD, k_lusgs_sweep<TB, TV, true><<<grid_for(count, SWEEP_THREADS), SWEEP_THREADS, 0, st>>>(
                                     m, (const TB*)h.blk, (const TB*)h.rD, (const TV*)h.kw, fwd, nullptr, order,
                                     count, m.sweep_ticket, &h.ks->status, spin_limit));
  ICS_CUDA(cudaGetLastError());
}

// LU-SGS sweeps on an FP64 vector with the given off-diagonal slots (factored
// FP32 or 25-entry FP64 storage) and scalar diagonal: the preconditioner of
// the matrix-free Krylov solves (k_krylov.cu), which transposes the blocks
// for the adjoint system
void lusgs_with(Handle& h, const void* blk, const void* rD, bool fp32, double* r) {
  if (fp32)
    lusgs_t<float, double>(h, r, (const float*)blk, (const float*)rD);
  else
    lusgs_t<double, double>(h, r, (const double*)blk, (const double*)rD);
  ICS_CUDA(cudaGetLastError());
}

bool fused_operator(Handle& h, const void* x, void* w, void* vout) {
  if (prec(h) == ICS_PREC_MIXED)
    return fused_op_t<float, float>(h, (const float*)x, (float*)w, (float*)vout);
  return fused_op_t<double, double>(h, (const double*)x, (double*)w, (double*)vout);
}

void sweep_probe(Handle& h, const int* order, int count, int spin_limit) {
  if (prec(h) == ICS_PREC_MIXED)
    sweep_probe_t<float, float>(h, order, count, spin_limit);
  else
    sweep_probe_t<double, double>(h, order, count, spin_limit);
}

void spmv(Handle& h, const void* x, void* y) {
  if (prec(h) == ICS_PREC_MIXED)
    spmv_t<float, float>(h, (const float*)x, (float*)y);
  else
    spmv_t<double, double>(h, (const double*)x, (double*)y);
  ICS_CUDA(cudaGetLastError());
}

int precondition(Handle& h, void* r) {
  if (prec(h) == ICS_PREC_MIXED)
    precondition_t<float, float>(h, (float*)r);
  else
    precondition_t<double, double>(h, (double*)r);
  ICS_CUDA(cudaGetLastError());
  return ICS_OK;
}

void to_vec(Handle& h, const double* src, void* dst) {
  const long n = 5L * h.m.N;
  if (prec(h) == ICS_PREC_MIXED)
    ICS_LAUNCH(h, ICS_K_VECTOR, k_cast<double, float><<<REDUCE_BLOCKS, RB, 0, h.stream>>>(n, src, (float*)dst));
  else
    ICS_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
}

void from_vec(Handle& h, const void* src, double* dst) {
  const long n = 5L * h.m.N;
  if (prec(h) == ICS_PREC_MIXED)
    ICS_LAUNCH(h, ICS_K_VECTOR, k_cast<float, double><<<REDUCE_BLOCKS, RB, 0, h.stream>>>(n, (const float*)src, dst));
  else
    ICS_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
}

// ----------------------------------------------------------------- GMRES
// residualsIO of the coupled system: initial and final L1 residuals per
// instance and equation, [5*J + k]
struct ResIO {
  std::vector<double> init, fin;
  int nIter = 0;
};

// coupledMatrix::solver::stop (coupledMatrixSolver.C:198-221) over every entry
static bool stop_test(const Handle& h, const ResIO& r) {
  const ics_config& c = h.cfg.c;
  if (r.nIter < c.min_iter) return false;
  double mx = -VGREAT, mrel = -VGREAT;
  for (double v : r.fin) mx = fmax(mx, v);
  for (int J = 0; J < h.m.nInst; ++J) {
    const double* in = &r.init[5 * J];
    const double* fi = &r.fin[5 * J];
    mrel = fmax(mrel, fi[0] / (in[0] + ROOTVSMALL));
    mrel = fmax(mrel, fi[4] / (in[4] + ROOTVSMALL));
    for (int k = 0; k < 3; ++k)
      if (h.m.solD[k] == 1) mrel = fmax(mrel, fi[1 + k] / (in[1 + k] + ROOTVSMALL));
  }
  return r.nIter >= c.max_iter || mx < c.tolerance || mrel < c.rel_tol;
}

// grid of the per-instance reductions: the instances share REDUCE_BLOCKS
static dim3 inst_grid(const Handle& h) {
  const int bx = REDUCE_BLOCKS / h.m.nInst;
  return dim3(bx < 1 ? 1 : bx, h.m.nInst);
}

// final L1 residuals from the per-instance sums in h.ksHost->res; false when
// any is not finite
static bool final_residuals(const Handle& h, const std::vector<double>& nf, ResIO& r) {
  bool finite = true;
  for (int J = 0; J < h.m.nInst; ++J) {
    const double* rs = h.ksHost->res + 5 * J;
    double* fi = &r.fin[5 * J];
    fi[0] = rs[0] / nf[3 * J];
    fi[4] = rs[4] / nf[3 * J + 1];
    for (int k = 0; k < 3; ++k) fi[1 + k] = h.m.solD[k] == -1 ? 0.0 : rs[1 + k] / nf[3 * J + 2];
    for (int k = 0; k < 5; ++k) finite = finite && std::isfinite(fi[k]);
  }
  return finite;
}

// Norm factors of coupledMatrixSolver (gmres.C:812-850): sum |A (W - avg W)| +
// |b| per equation (vector magnitude for rhoU), and the initial L1 residuals,
// each per instance (gAverage and gSum per field).
template <typename TB, typename TV>
static void norm_factors_t(Handle& h, std::vector<double>& nf, ResIO& r) {
  const int N = h.m.N, Nc = h.m.Nc, nI = h.m.nInst;
  cudaStream_t st = h.stream;
  KrylovScalars* ks = h.ks;
  TV* w = (TV*)h.kw;
  TV* t = (TV*)h.kt;
  const dim3 g = inst_grid(h);
  ICS_CUDA(cudaMemsetAsync(&ks->status, 0, sizeof(int), st));
  ICS_LAUNCH(h, ICS_K_VECTOR, k_wsum<<<g, RB, 0, st>>>(Nc, h.W, h.partials, h.counter, ks->avg));
  ICS_LAUNCH(h, ICS_K_SCALAR, k_avg<<<1, 1, 0, st>>>(ks, Nc, nI));
  ICS_LAUNCH(h, ICS_K_VECTOR, k_wmavg<TV><<<grid_for(N, 256), 256, 0, st>>>(N, Nc, h.W, ks, w));
  spmv_t<TB, TV>(h, w, t);
  ICS_LAUNCH(h, ICS_K_VECTOR, k_normfac<TV><<<g, RB, 0, st>>>(Nc, h.src, t, h.partials, h.counter, ks->nfr));
  ICS_CUDA(cudaMemcpyAsync(h.ksHost->nfr, ks->nfr, 8 * nI * sizeof(double), cudaMemcpyDeviceToHost, st));
  ICS_CUDA(cudaStreamSynchronize(st));
  nf.assign(3 * nI, 0.0);
  r.init.assign(5 * nI, 0.0);
  r.nIter = 0;
  for (int J = 0; J < nI; ++J) {
    const double* q = h.ksHost->nfr + 8 * J;
    for (int k = 0; k < 3; ++k) nf[3 * J + k] = q[k] + VSMALL;
    double* in = &r.init[5 * J];
    in[0] = q[3] / nf[3 * J];
    in[1] = q[4] / nf[3 * J + 2];
    in[2] = q[5] / nf[3 * J + 2];
    in[3] = q[6] / nf[3 * J + 2];
    in[4] = q[7] / nf[3 * J + 1];
  }
  r.fin = r.init;
}

// x_new = D^-1 (b - (A - D) x_old): one block-Jacobi sweep (JacobiSmoother::smooth)
template <typename TB, typename TV>
__global__ void __launch_bounds__(128) k_jacobi_sweep(DevMesh m, const TB* __restrict__ blk,
                                                      const TB* __restrict__ inv, const double* __restrict__ b,
                                                      const TV* __restrict__ xo, TV* __restrict__ xn) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int s = c >> 5, lane = c & 31;
  TV acc[5] = {TV(0), TV(0), TV(0), TV(0), TV(0)};
  const int base = m.slot_base[s];
  const TV g = TV(m.gamma);
  for (int t = 0; t < m.nslot[c]; ++t) {
    const int col = m.scol[(base + t) * 32 + lane];
    TV xj[5], y[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xj[k] = xo[5 * col + k];
    SlotBlock<TB> Bk;
    Bk.load(blk, base + t, lane);
    Bk.mv(g, xj, y);
    if (m.vjslot) vj_sub<TB>(m, base + t, lane, col, xj, y);
#pragma unroll
    for (int i = 0; i < 5; ++i) acc[i] += y[i];
  }
  TV r[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) r[k] = -(acc[k] - TV(b[5 * c + k]));
  const TB* D = inv + (size_t)s * 25 * 32 + lane;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    TV a = TV(0);
#pragma unroll
    for (int j = 0; j < 5; ++j) a += TV(D[(5 * i + j) * 32]) * r[j];
    xn[5 * c + i] = a;
  }
}

// smoothSolverCoupled::solveDelta (smoothSolverCoupled.C:369-515)
template <typename TB, typename TV>
static int smooth_t(Handle& h, ResIO& p) {
  const int N = h.m.N;
  const long n5 = 5L * N;
  cudaStream_t st = h.stream;
  KrylovScalars* ks = h.ks;
  std::vector<double> nf;
  norm_factors_t<TB, TV>(h, nf, p);
  TV* x = (TV*)h.kx;
  TV* y = (TV*)h.kb;
  TV* t = (TV*)h.kt;
  TV* r = (TV*)h.kw;
  ICS_CUDA(cudaMemsetAsync(x, 0, n5 * sizeof(TV), st));
  bool finite = true;
  do {
    for (int s = 0; s < h.cfg.c.n_sweeps; ++s) {
      ICS_LAUNCH(h, ICS_K_JACOBI,
                 k_jacobi_sweep<TB, TV><<<grid_for(N, 128), 128, 0, st>>>(h.m, (const TB*)h.blk, (const TB*)h.dginv,
                                                                          h.src, x, y));
      TV* tmp = x;
      x = y;
      y = tmp;
    }
    spmv_t<TB, TV>(h, x, t);
    ICS_LAUNCH(h, ICS_K_VECTOR,
               k_resid<TV><<<inst_grid(h), RB, 0, st>>>(h.m.Nc, h.src, t, r, h.partials, h.counter, ks->res));
    ICS_CUDA(cudaGetLastError());
    ICS_CUDA(cudaMemcpyAsync(h.ksHost->res, ks->res, 5 * h.m.nInst * sizeof(double), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaStreamSynchronize(st));
    finite = final_residuals(h, nf, p);
    p.nIter += h.cfg.c.n_sweeps;
    if (!finite) break;
  } while (!stop_test(h, p));
  ICS_LAUNCH(h, ICS_K_VECTOR,
             k_to_dW<TV><<<grid_for(N, 256), 256, 0, st>>>(N, x, h.dW, h.m.solD[0], h.m.solD[1], h.m.solD[2]));
  ICS_CUDA(cudaGetLastError());
  return finite ? ICS_OK : ICS_ERR_NONFINITE;
}


template <typename TB, typename TV>
static int gmres_t(Handle& h, ResIO& p) {
  const int N = h.m.N, m = h.cfg.c.n_directions;
  const long n5 = 5L * N;
  const long vs = (long)kstride(h);
  cudaStream_t st = h.stream;
  KrylovScalars* ks = h.ks;
  TV* V = (TV*)h.kv;
  TV* w = (TV*)h.kw;
  TV* x = (TV*)h.kx;
  TV* t = (TV*)h.kt;
  double* red = ks->red;
  std::vector<double> nf;
  norm_factors_t<TB, TV>(h, nf, p);
  // r = b, x = 0
  ICS_CUDA(cudaMemsetAsync(x, 0, n5 * sizeof(TV), st));
  to_vec(h, h.src, w);
  int status = ICS_OK;
  // one restart cycle: every scalar it needs lives in device memory, so the
  // same launch sequence can be captured once and replayed per cycle
  auto cycle = [&]() {
    precondition_t<TB, TV>(h, w);
    ICS_LAUNCH(h, ICS_K_MGS,
               k_mgs<TV><<<h.tuneMgsBlocks, RB, 0, st>>>(n5, w, nullptr, nullptr, nullptr, &ks->status, h.partials,
                                                       h.counter, red, ks, 1, 0, m));
    // with the fused operator the step's normalisation is folded into it and
    // the unnormalised vector alternates between two buffers (w, t); the
    // cycle's residual goes back to w
    const bool fused = fused_op_available<TB, TV>(h);
    TV* wb[2] = {w, t};
    TV* wc = w;
    for (int i = 0; i < m; ++i) {
      TV* vi = V + (size_t)i * vs;
      if (fused) {
        fused_op_t<TB, TV>(h, wb[i & 1], wb[(i + 1) & 1], vi);
        wc = wb[(i + 1) & 1];
      } else {
        ICS_LAUNCH(h, ICS_K_VECTOR, k_scale<TV><<<REDUCE_BLOCKS, RB, 0, st>>>(n5, wc, vi, ks));
        spmv_t<TB, TV>(h, vi, wc);
        precondition_t<TB, TV>(h, wc);
      }
      for (int j = 0; j <= i; ++j) {
        const TV* vprev = j > 0 ? V + (size_t)(j - 1) * vs : nullptr;
        const double* hprev = j > 0 ? &ks->H[(j - 1) * m + i] : nullptr;
        ICS_LAUNCH(h, ICS_K_MGS,
                   k_mgs<TV><<<h.tuneMgsBlocks, RB, 0, st>>>(n5, wc, vprev, hprev, V + (size_t)j * vs, &ks->status,
                                                           h.partials, h.counter, &ks->H[j * m + i], ks, 0, i, m));
      }
      ICS_LAUNCH(h, ICS_K_MGS,
                 k_mgs<TV><<<h.tuneMgsBlocks, RB, 0, st>>>(n5, wc, vi, &ks->H[i * m + i], nullptr, &ks->status,
                                                         h.partials, h.counter, &red[1], ks, 2, i, m));
    }
    ICS_LAUNCH(h, ICS_K_SCALAR, k_backsub<<<1, 1, 0, st>>>(ks, m));
    ICS_LAUNCH(h, ICS_K_VECTOR, k_xupdate<TV><<<REDUCE_BLOCKS, RB, 0, st>>>(n5, x, V, ks, m, vs));
    spmv_t<TB, TV>(h, x, t);
    ICS_LAUNCH(h, ICS_K_VECTOR,
               k_resid<TV><<<inst_grid(h), RB, 0, st>>>(h.m.Nc, h.src, t, w, h.partials, h.counter, ks->res));
  };
  // the captured launches hold DevMesh by value: the non-LF viscous block
  // parts (m.vjslot) are part of the key
  const int key = (h.m.vjslot ? 10000000 : 0) + h.cfg.c.preconditioner * 100000 + prec(h) * 1000 + m;
  const bool useGraph = !h.prof;  // per-launch event timing needs direct launches
  if (useGraph && h.cycleKey != key) {
    drop_graphs(h);
    cudaGraph_t g = nullptr;
    const long long before = h.launches;
    ICS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cycle();
    ICS_CUDA(cudaStreamEndCapture(st, &g));
    ICS_CUDA(cudaGraphInstantiate(&h.cycleExec, g, 0));
    ICS_CUDA(cudaGraphDestroy(g));
    h.cycleLaunches = h.launches - before;
    h.launches = before;  // captured, not executed
    h.cycleKey = key;
  }
  do {
    if (useGraph) {
      ICS_CUDA(cudaGraphLaunch(h.cycleExec, st));
      h.launches += h.cycleLaunches;
    } else {
      cycle();
    }
    ICS_CUDA(cudaGetLastError());
    ICS_CUDA(cudaMemcpyAsync(h.ksHost->res, ks->res, 5 * h.m.nInst * sizeof(double), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaMemcpyAsync(&h.ksHost->status, &ks->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaStreamSynchronize(st));
    if (h.ksHost->status) {
      status = (h.ksHost->status & 8) ? ICS_ERR_TIMEOUT
                                      : ((h.ksHost->status & 4) ? ICS_ERR_NONFINITE : ICS_ERR_BREAKDOWN);
      p.nIter++;
      break;
    }
    const bool finite = final_residuals(h, nf, p);
    p.nIter++;
    if (!finite) {
      status = ICS_ERR_NONFINITE;
      break;
    }
  } while (!stop_test(h, p));
  ICS_LAUNCH(h, ICS_K_VECTOR, k_to_dW<TV><<<grid_for(N, 256), 256, 0, st>>>(N, x, h.dW, h.m.solD[0], h.m.solD[1], h.m.solD[2]));
  ICS_CUDA(cudaGetLastError());
  return status;
}

int gmres_solve(Handle& h, ics_solver_perf* perf, std::vector<double>& initRes) {
  ResIO r;
  int st;
  if (h.cfg.c.solver == ICS_SOLVER_SMOOTH)
    st = prec(h) == ICS_PREC_MIXED ? smooth_t<float, float>(h, r) : smooth_t<double, double>(h, r);
  else
    st = prec(h) == ICS_PREC_MIXED ? gmres_t<float, float>(h, r) : gmres_t<double, double>(h, r);
  // the C ABI's summary: maximum over instances per equation
  memset(perf, 0, sizeof(*perf));
  for (int k = 0; k < 5; ++k) {
    perf->init_res[k] = -VGREAT;
    perf->final_res[k] = -VGREAT;
    for (int J = 0; J < h.m.nInst; ++J) {
      perf->init_res[k] = fmax(perf->init_res[k], r.init[5 * J + k]);
      perf->final_res[k] = fmax(perf->final_res[k], r.fin[5 * J + k]);
    }
  }
  perf->n_iterations = r.nIter;
  perf->converged = st == ICS_OK;
  initRes = r.init;
  return st;
}

// ------------------------------------------------------------ autotuner
// Times the Krylov-side launch choices on the handle's assembled system with
// CUDA events on its stream (median of three runs each, after a warm-up):
// the MGS step's grid, and the fused LU-SGS operator against SpMV plus
// separate sweeps.  Sets the fastest; the arithmetic of every choice is the
// same up to the order of the sums.
template <typename TB, typename TV>
static void autotune_linalg_t(Handle& h, std::vector<std::pair<std::string, double>>& log) {
  cudaStream_t st = h.stream;
  const long n5 = 5L * h.m.N;
  TV* V = (TV*)h.kv;
  TV* w = (TV*)h.kw;
  TV* t = (TV*)h.kt;
  cudaEvent_t e0, e1;
  ICS_CUDA(cudaEventCreate(&e0));
  ICS_CUDA(cudaEventCreate(&e1));
  auto timed = [&](auto&& fn) {
    fn();
    double best[5];
    for (int r = 0; r < 5; ++r) {
      ICS_CUDA(cudaEventRecord(e0, st));
      fn();
      ICS_CUDA(cudaEventRecord(e1, st));
      ICS_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      ICS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best[r] = ms;
    }
    std::sort(best, best + 5);
    return best[2];
  };
  // operands: w = b, v_0 = b (a step of the cycle's Gram-Schmidt)
  to_vec(h, h.src, w);
  to_vec(h, h.src, V);
  KrylovScalars* ks = h.ks;
  const int m = h.cfg.c.n_directions;
  int bestBlocks = h.tuneMgsBlocks;
  double bestMs = 1e300;
  // the cycle's steps: w -= h v_{j-1}, then w . v_j over the m basis vectors
  // in turn (their working set exceeds L2 as in the cycle; one launch alone
  // is too short to time); h = 0 keeps w
  const long vs = (long)kstride(h);
  for (int j = 1; j < m; ++j) to_vec(h, h.src, V + (size_t)j * vs);
  ICS_CUDA(cudaMemsetAsync(&ks->red[15], 0, sizeof(double), st));
  ICS_CUDA(cudaMemsetAsync(&ks->status, 0, sizeof(int), st));
  for (int blocks : {152, 304, 456, 608}) {
    const double ms = timed([&]() {
      for (int j = 0; j < m; ++j)
        k_mgs<TV><<<blocks, RB, 0, st>>>(n5, w, V + (size_t)((j + m - 1) % m) * vs, &ks->red[15],
                                          V + (size_t)j * vs, &ks->status, h.partials, h.counter, &ks->red[14], ks,
                                          0, 0, m);
    });
    log.emplace_back("mgs_blocks_" + std::to_string(blocks), ms);
    if (ms < bestMs) bestMs = ms, bestBlocks = blocks;
  }
  h.tuneMgsBlocks = bestBlocks;
  ICS_CUDA(cudaMemsetAsync(&ks->status, 0, sizeof(int), st));
  h.tuneFused = 1;
  if (fused_op_available<TB, TV>(h)) {
    const double fused = timed([&]() { fused_op_t<TB, TV>(h, V, w); });
    const double split = timed([&]() {
      spmv_t<TB, TV>(h, V, t);
      precondition_t<TB, TV>(h, t);
    });
    log.emplace_back("operator_fused", fused);
    log.emplace_back("operator_spmv_then_lusgs", split);
    h.tuneFused = fused <= split ? 1 : 0;
  }
  // rows per thread of the reverse level sweeps, timed on the whole LU-SGS
  double revMs[3] = {0, 0, 0};
  for (int rows : {1, 2}) {
    h.tuneRevRows = rows;
    revMs[rows] = timed([&]() {
      to_vec(h, h.src, t);
      precondition_t<TB, TV>(h, t);
    });
    log.emplace_back("reverse_rows_" + std::to_string(rows), revMs[rows]);
  }
  h.tuneRevRows = revMs[2] < revMs[1] ? 2 : 1;
  ICS_CUDA(cudaEventDestroy(e0));
  ICS_CUDA(cudaEventDestroy(e1));
  ICS_CUDA(cudaGetLastError());
}

void autotune_linalg(Handle& h, std::vector<std::pair<std::string, double>>& log) {
  if (prec(h) == ICS_PREC_MIXED)
    autotune_linalg_t<float, float>(h, log);
  else
    autotune_linalg_t<double, double>(h, log);
}

// sum of a device array (deterministic fixed-order reduction)
double device_sum(Handle& h, const double* a, int n) {
  ICS_LAUNCH(h, ICS_K_VECTOR, k_sumsq<<<REDUCE_BLOCKS, RB, 0, h.stream>>>(n, a, h.partials, h.counter, &h.ks->red[8]));
  double v = 0;
  ICS_CUDA(cudaMemcpyAsync(&v, &h.ks->red[8], sizeof(double), cudaMemcpyDeviceToHost, h.stream));
  ICS_CUDA(cudaStreamSynchronize(h.stream));
  return v;
}

// rho L2 residual: sqrt(sum (div(phi) V)^2) from the per-cell squares
double rho_l2(Handle& h) {
  ICS_LAUNCH(h, ICS_K_VECTOR, k_sumsq<<<REDUCE_BLOCKS, RB, 0, h.stream>>>(h.m.N, h.scratch, h.partials, h.counter, &h.ks->l2));
  double v = 0;
  ICS_CUDA(cudaMemcpyAsync(&v, &h.ks->l2, sizeof(double), cudaMemcpyDeviceToHost, h.stream));
  ICS_CUDA(cudaStreamSynchronize(h.stream));
  return std::sqrt(v);
}

// ------------------------------------------------------ passive scalar
// The 1x0 coupled system of the scalar transport (same GMRES, LU-SGS and
// norm factors as the flow's, one equation): 1x1 sliced-ELL blocks, FP64.
__global__ void __launch_bounds__(128) k_s_spmv(DevMesh m, const double* __restrict__ blk,
                                                const double* __restrict__ dg, const double* __restrict__ x,
                                                double* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int s = c >> 5, lane = c & 31;
  double acc = dg[c] * x[c];
  const int base = m.slot_base[s];
  for (int t = 0; t < m.nslot[c]; ++t) {
    const int col = m.scol[(base + t) * 32 + lane];
    acc += blk[(size_t)(base + t) * 32 + lane] * x[col];
  }
  y[c] = acc;
}

__device__ __forceinline__ void s_fwd_row(const DevMesh& m, const double* __restrict__ blk,
                                          const double* __restrict__ rD, double* __restrict__ r, int c, bool scale) {
  const int s = c >> 5, lane = c & 31;
  const int base = m.slot_base[s];
  double acc = r[c];
  for (int t = 0; t < m.nlow[c]; ++t) {
    const int col = m.scol[(base + t) * 32 + lane];
    acc -= blk[(size_t)(base + t) * 32 + lane] * (rD[col] * r[col]);
  }
  r[c] = scale ? rD[c] * acc : acc;
}

__device__ __forceinline__ void s_rev_row(const DevMesh& m, const double* __restrict__ blk,
                                          const double* __restrict__ rD, double* __restrict__ r, int c) {
  const int s = c >> 5, lane = c & 31;
  const int base = m.slot_base[s];
  double acc = r[c];
  for (int t = m.nslot[c] - 1; t >= m.nlow[c]; --t) {
    const int col = m.scol[(base + t) * 32 + lane];
    acc -= blk[(size_t)(base + t) * 32 + lane] * r[col];
  }
  r[c] = rD[c] * acc;
}

template <int MODE>
__global__ void __launch_bounds__(128) k_s_lusgs_level(DevMesh m, const double* __restrict__ blk,
                                                       const double* __restrict__ rD, double* __restrict__ r,
                                                       const int* __restrict__ cells, int start, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int c = cells ? cells[start + i] : start + i;
  if (MODE == 1)
    s_rev_row(m, blk, rD, r, c);
  else
    s_fwd_row(m, blk, rD, r, c, MODE == 2);
}

template <bool FWD>
__global__ void __launch_bounds__(1024) k_s_lusgs_block(DevMesh m, const double* __restrict__ blk,
                                                        const double* __restrict__ rD, double* __restrict__ r,
                                                        const int* __restrict__ cells, const int* __restrict__ lptr,
                                                        int nlev) {
  for (int l = 0; l < nlev; ++l) {
    for (int i = lptr[l] + threadIdx.x; i < lptr[l + 1]; i += blockDim.x) {
      if (FWD)
        s_fwd_row(m, blk, rD, r, cells[i], false);
      else
        s_rev_row(m, blk, rD, r, cells[i]);
    }
    __syncthreads();
  }
}

__global__ void k_s_jacobi(int N, const double* __restrict__ dg, double* __restrict__ r) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < N) r[c] /= dg[c];
}

// out[0] = sum w
__global__ void __launch_bounds__(RB) k_s_sum(int N, const double* __restrict__ w, double* __restrict__ partials,
                                              unsigned int* __restrict__ counter, double* __restrict__ out) {
  double acc[1] = {0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) acc[0] += w[c];
  reduce_finish<1>(acc, partials, counter, out);
}

__global__ void k_s_wmavg(int N, const double* __restrict__ w, const double* __restrict__ sum,
                          double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < N) out[c] = w[c] - sum[0] / N;
}

// out[0] = sum |t| + |b|, out[1] = sum |b|
__global__ void __launch_bounds__(RB) k_s_normfac(int N, const double* __restrict__ b, const double* __restrict__ t,
                                                  double* __restrict__ partials, unsigned int* __restrict__ counter,
                                                  double* __restrict__ out) {
  double acc[2] = {0.0, 0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    acc[0] += fabs(t[c]) + fabs(b[c]);
    acc[1] += fabs(b[c]);
  }
  reduce_finish<2>(acc, partials, counter, out);
}

// r = b - t, out[0] = sum |r|
__global__ void __launch_bounds__(RB) k_s_resid(int N, const double* __restrict__ b, const double* __restrict__ t,
                                                double* __restrict__ r, double* __restrict__ partials,
                                                unsigned int* __restrict__ counter, double* __restrict__ out) {
  double acc[1] = {0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    const double v = b[c] - t[c];
    r[c] = v;
    acc[0] += fabs(v);
  }
  reduce_finish<1>(acc, partials, counter, out);
}

// scalar cyclic interfaces: y_c += sum over c's cyclic faces of a_f x_partner
// (a_f in the upper slot of the scalar face coefficients)
__global__ void k_s_cyc_mv(DevMesh m, const double* __restrict__ sface, int FB, const double* __restrict__ x,
                           double* __restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m.ncrow) return;
  const int c = m.cyc_row[r];
  double acc = y[c];
  for (int e = m.cyc_ptr[r]; e < m.cyc_ptr[r + 1]; ++e) {
    const int b = m.cyc_face[e];
    acc += sface[FB + m.F + b] * x[m.bpartner[b]];
  }
  y[c] = acc;
}

static void s_spmv(Handle& h, const double* x, double* y) {
  ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_spmv<<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m, h.sblk, h.sdg, x, y));
  if (h.m.ncrow)
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_cyc_mv<<<grid_for(h.m.ncrow, 128), 128, 0, h.stream>>>(h.m, h.sface, h.m.F + h.m.B,
                                                                                            x, y));
}

static void s_precondition(Handle& h, double* r) {
  const DevMesh& m = h.m;
  const int pc = h.cfg.c.preconditioner;
  if (pc == ICS_PC_JACOBI) {
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_jacobi<<<grid_for(m.N, 256), 256, 0, h.stream>>>(m.N, h.sdg, r));
    return;
  }
  if (pc != ICS_PC_LUSGS) return;
  if ((long)m.N < 2048L * m.nfl) {
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_lusgs_block<true><<<1, 1024, 0, h.stream>>>(m, h.sblk, h.srD, r, m.fl_cells,
                                                                                  m.fl_lptr, m.nfl));
  } else {
    for (int l = 1; l < m.nfl; ++l) {  // level 0 has no lower neighbours
      const int a = m.fl_ptr[l], cnt = m.fl_ptr[l + 1] - a;
      const bool contig = m.fl_cstart[l] >= 0;
      ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_lusgs_level<0><<<grid_for(cnt, 128), 128, 0, h.stream>>>(
                                       m, h.sblk, h.srD, r, contig ? nullptr : m.fl_cells,
                                       contig ? m.fl_cstart[l] : a, cnt));
    }
  }
  if ((long)m.N < 2048L * m.nrl) {
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_lusgs_block<false><<<1, 1024, 0, h.stream>>>(m, h.sblk, h.srD, r, m.rl_cells,
                                                                                   m.rl_lptr, m.nrl));
  } else {
    for (int l = 0; l < m.nrl; ++l) {
      const int a = m.rl_ptr[l], cnt = m.rl_ptr[l + 1] - a;
      const bool contig = m.rl_cstart[l] >= 0;
      ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_lusgs_level<1><<<grid_for(cnt, 128), 128, 0, h.stream>>>(
                                       m, h.sblk, h.srD, r, contig ? nullptr : m.rl_cells,
                                       contig ? m.rl_cstart[l] : a, cnt));
    }
  }
}

// gmres::solveDelta on the scalar system: b = h.ssrc, norm factors from the
// previous-iteration rhoS, increment in dx
int scalar_gmres(Handle& h, double* dx, ics_solver_perf* perf) {
  const int N = h.m.N, m = h.cfg.c.n_directions;
  cudaStream_t st = h.stream;
  KrylovScalars* ks = h.ks;
  const long vs = ((long)N + 63) / 64 * 64;
  double* V = (double*)h.kv;
  double* w = (double*)h.kw;
  double* t = (double*)h.kt;
  double* red = ks->red;
  ICS_CUDA(cudaMemsetAsync(&ks->status, 0, sizeof(int), st));
  ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_sum<<<REDUCE_BLOCKS, RB, 0, st>>>(N, h.srhoS, h.partials, h.counter, &red[2]));
  ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_wmavg<<<grid_for(N, 256), 256, 0, st>>>(N, h.srhoS, &red[2], w));
  s_spmv(h, w, t);
  ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_normfac<<<REDUCE_BLOCKS, RB, 0, st>>>(N, h.ssrc, t, h.partials, h.counter, &red[3]));
  double hv[2];
  ICS_CUDA(cudaMemcpyAsync(hv, &red[3], 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  ICS_CUDA(cudaStreamSynchronize(st));
  const double nf = hv[0] + VSMALL;
  memset(perf, 0, sizeof(*perf));
  perf->init_res[0] = perf->final_res[0] = hv[1] / nf;
  ICS_CUDA(cudaMemsetAsync(dx, 0, N * sizeof(double), st));
  ICS_CUDA(cudaMemcpyAsync(w, h.ssrc, N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  const ics_config& cf = h.cfg.c;
  int status = ICS_OK;
  while (true) {
    s_precondition(h, w);
    ICS_LAUNCH(h, ICS_K_MGS, k_mgs<double><<<h.tuneMgsBlocks, RB, 0, st>>>(N, w, nullptr, nullptr, nullptr, &ks->status,
                                                                       h.partials, h.counter, red, ks, 1, 0, m));
    for (int i = 0; i < m; ++i) {
      double* vi = V + (size_t)i * vs;
      ICS_LAUNCH(h, ICS_K_VECTOR, k_scale<double><<<REDUCE_BLOCKS, RB, 0, st>>>(N, w, vi, ks));
      s_spmv(h, vi, w);
      s_precondition(h, w);
      for (int j = 0; j <= i; ++j) {
        const double* vprev = j > 0 ? V + (size_t)(j - 1) * vs : nullptr;
        const double* hprev = j > 0 ? &ks->H[(j - 1) * m + i] : nullptr;
        ICS_LAUNCH(h, ICS_K_MGS,
                   k_mgs<double><<<h.tuneMgsBlocks, RB, 0, st>>>(N, w, vprev, hprev, V + (size_t)j * vs, &ks->status,
                                                            h.partials, h.counter, &ks->H[j * m + i], ks, 0, i, m));
      }
      ICS_LAUNCH(h, ICS_K_MGS, k_mgs<double><<<h.tuneMgsBlocks, RB, 0, st>>>(N, w, vi, &ks->H[i * m + i], nullptr,
                                                                         &ks->status, h.partials, h.counter, &red[1],
                                                                         ks, 2, i, m));
    }
    ICS_LAUNCH(h, ICS_K_SCALAR, k_backsub<<<1, 1, 0, st>>>(ks, m));
    ICS_LAUNCH(h, ICS_K_VECTOR, k_xupdate<double><<<REDUCE_BLOCKS, RB, 0, st>>>(N, dx, V, ks, m, vs));
    s_spmv(h, dx, t);
    ICS_LAUNCH(h, ICS_K_PASSIVE, k_s_resid<<<REDUCE_BLOCKS, RB, 0, st>>>(N, h.ssrc, t, w, h.partials, h.counter,
                                                                         &red[5]));
    double rs = 0;
    int stt = 0;
    ICS_CUDA(cudaMemcpyAsync(&rs, &red[5], sizeof(double), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaMemcpyAsync(&stt, &ks->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaStreamSynchronize(st));
    perf->n_iterations++;
    if (stt) {
      status = (stt & 4) ? ICS_ERR_NONFINITE : ICS_ERR_BREAKDOWN;
      break;
    }
    perf->final_res[0] = rs / nf;
    if (!std::isfinite(perf->final_res[0])) {
      status = ICS_ERR_NONFINITE;
      break;
    }
    if (perf->n_iterations < cf.min_iter) continue;
    const double rel = perf->final_res[0] / (perf->init_res[0] + ROOTVSMALL);
    if (perf->n_iterations >= cf.max_iter || perf->final_res[0] < cf.tolerance || rel < cf.rel_tol) break;
  }
  perf->converged = status == ICS_OK;
  ICS_CUDA(cudaGetLastError());
  return status;
}

}  // namespace ics
