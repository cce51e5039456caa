// Independent cases stacked in one handle: the batch of many small cases as a
// leading dimension.
//
// The handle's mesh is the disjoint union of the cases' meshes (case k owns
// cells start[k] .. start[k+1]-1; no face joins two cases), so every
// cell- and face-parallel kernel of the pseudo iteration (fields, gradients,
// fluxes, cell residual, Jacobian rows, SpMV, LU-SGS levels, update) already
// treats each case exactly as a handle of its own would, and runs once for
// all of them.  What couples the cells of one system are the scalars of its
// GMRES (gmres.C:772-1107): the dot products and norms, the Hessenberg
// matrix, the Givens rotations, the back substitution, the stop test
// (coupledMatrixSolver.C:198-221) and the norm factors (gmres.C:812-850).
// Here each of those is per case:
//   * every reduction runs over segments of at most SEG_CELLS cells that
//     never straddle two cases; the last segment of a case to finish folds
//     the case's partial sums in segment order (a per-case last-block-done
//     tree), so a case's sums depend only on its own cells and sizes, not on
//     the other cases in the stack;
//   * the Krylov scalars (H, c, s, bh, y, beta) live per case in device
//     memory and the per-case kernels read them there, so one restart cycle
//     is one launch sequence for all cases, captured once as a CUDA graph;
//   * the host reads every case's L1 residuals after a cycle and applies the
//     stop test per case; a case that has stopped (or broken down) is marked
//     inactive and its correction is left as it stands while the others go
//     on.
// The LU-SGS preconditioner, the SpMV and the fused operator passes are the
// handle's own (union) kernels: their rows only read rows of the same case, and
// the fused passes scale each row by its own case's Krylov norm.
#include <algorithm>
#include <cmath>

#include "ics_internal.cuh"

namespace ics {

namespace {

constexpr int SEG_CELLS = 1024;  // cells per reduction segment (5120 vector entries)
constexpr int CB = 256;          // threads per segment block
constexpr int PSTRIDE = 8;       // partial sums per segment
constexpr int HSTRIDE = MAX_DIRS * MAX_DIRS;

__device__ __forceinline__ bool case_on(const CaseDev& D, int c) { return D.active[c] && D.status[c] == 0; }

// Block-sum NV values, store them as this segment's partials, and on the
// last segment of case c to arrive fold the case's partials in segment order
// into out[0..NV).  True on thread 0 of that block.
template <int NV>
__device__ __forceinline__ bool case_finish(const CaseDev& D, int c, double (&v)[NV], double* __restrict__ out) {
  __shared__ double sm[CB / 32][NV];
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
  const int s0 = D.caseSeg[c], ns = D.caseSeg[c + 1] - s0;
  if (threadIdx.x == 0) {
    for (int k = 0; k < NV; ++k) {
      double s = 0;
      for (int w = 0; w < CB / 32; ++w) s += sm[w][k];
      D.partials[(size_t)blockIdx.x * PSTRIDE + k] = s;
    }
    __threadfence();
    const unsigned t = atomicAdd(&D.counter[c], 1u);
    amLast = (t == (unsigned)ns - 1);
  }
  __syncthreads();
  if (!amLast) return false;
  __threadfence();
  const volatile double* vp = D.partials;
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  for (int b = threadIdx.x; b < ns; b += CB)
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] += vp[(size_t)(s0 + b) * PSTRIDE + k];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sm[warp][k] = x;  // thread 0 read sm before the barrier above
  }
  __syncthreads();
  if (threadIdx.x != 0) return false;
  for (int k = 0; k < NV; ++k) {
    double s = 0;
    for (int w = 0; w < CB / 32; ++w) s += sm[w][k];
    out[k] = s;
  }
  D.counter[c] = 0;
  return true;
}

__device__ __forceinline__ void case_givens(double h, double beta, double& c, double& s) {
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

// start of a cycle for case c: beta = |w|, bh = (beta, 0, ...)
__device__ void case_beta0(const CaseDev& D, int c) {
  const double beta = sqrt(D.red[2 * c]);
  D.beta[c] = beta;
  double* bh = D.bh + (size_t)c * (MAX_DIRS + 1);
  for (int i = 0; i <= D.m; ++i) bh[i] = 0.0;
  bh[0] = beta;
  if (!(beta > 0.0)) D.status[c] = isfinite(beta) ? 2 : 4;
}

// Hessenberg column i of case c: apply the previous rotations, make a new one
// (gmres.C:1013-1027, rotation gmres.C:44-69)
__device__ void case_hess(const CaseDev& D, int c, int i) {
  const int m = D.m;
  double* H = D.H + (size_t)c * HSTRIDE;
  double* cs = D.c + (size_t)c * MAX_DIRS;
  double* sn = D.s + (size_t)c * MAX_DIRS;
  double* bh = D.bh + (size_t)c * (MAX_DIRS + 1);
  const double beta = sqrt(D.red[2 * c + 1]);
  for (int j = 0; j < i; ++j) {
    const double Hji = H[j * m + i];
    H[j * m + i] = cs[j] * Hji - sn[j] * H[(j + 1) * m + i];
    H[(j + 1) * m + i] = sn[j] * Hji + cs[j] * H[(j + 1) * m + i];
  }
  case_givens(H[i * m + i], beta, cs[i], sn[i]);
  const double bhi = bh[i];
  bh[i] = cs[i] * bhi - sn[i] * bh[i + 1];
  bh[i + 1] = sn[i] * bhi + cs[i] * bh[i + 1];
  H[i * m + i] = cs[i] * H[i * m + i] - sn[i] * beta;
  D.beta[c] = beta;
}

// One pipelined modified Gram-Schmidt step per case (as the single-system
// k_mgs): w -= hprev vprev (when vprev), then the sum of w.vnext (or w.w) into
// H[outIdx] (outRed < 0) or red[outRed]; post 1 starts the cycle, post 2
// finishes Hessenberg column dir.
template <typename TV>
__global__ void __launch_bounds__(CB) k_cmgs(CaseDev D, TV* __restrict__ w, const TV* __restrict__ vprev,
                                             int hprevIdx, const TV* __restrict__ vnext, int outIdx, int outRed,
                                             int post, int dir) {
  const int c = D.segCase[blockIdx.x];
  const bool on = case_on(D, c);
  double acc[1] = {0.0};
  if (on) {
    const long e0 = 5L * D.segBeg[blockIdx.x], e1 = 5L * D.segEnd[blockIdx.x];
    const TV h = vprev ? TV(D.H[(size_t)c * HSTRIDE + hprevIdx]) : TV(0);
    TV t = TV(0);
    for (long e = e0 + threadIdx.x; e < e1; e += CB) {
      TV x = w[e];
      if (vprev) {
        x -= h * vprev[e];
        w[e] = x;
      }
      t += x * (vnext ? vnext[e] : x);
    }
    acc[0] = double(t);
  }
  double* out = outRed < 0 ? D.H + (size_t)c * HSTRIDE + outIdx : D.red + 2 * c + outRed;
  if (case_finish<1>(D, c, acc, out) && on) {
    if (post == 1)
      case_beta0(D, c);
    else if (post == 2)
      case_hess(D, c, dir);
  }
}

// v = w / beta of the segment's case
template <typename TV>
__global__ void __launch_bounds__(CB) k_cscale(CaseDev D, const TV* __restrict__ w, TV* __restrict__ v) {
  const int c = D.segCase[blockIdx.x];
  if (!case_on(D, c)) return;
  const TV beta = TV(D.beta[c]);
  const long e1 = 5L * D.segEnd[blockIdx.x];
  for (long e = 5L * D.segBeg[blockIdx.x] + threadIdx.x; e < e1; e += CB) v[e] = w[e] / beta;
}

// back substitution H y = bh per case (one thread per case)
__global__ void k_cbacksub(CaseDev D) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= D.n || !case_on(D, c)) return;
  const int m = D.m;
  const double* H = D.H + (size_t)c * HSTRIDE;
  const double* bh = D.bh + (size_t)c * (MAX_DIRS + 1);
  double* y = D.y + (size_t)c * MAX_DIRS;
  for (int i = m - 1; i >= 0; --i) {
    double sum = bh[i];
    for (int j = i + 1; j < m; ++j) sum -= H[i * m + j] * y[j];
    const double hii = H[i * m + i];
    const double st = hii >= 0 ? hii + VSMALL : hii - VSMALL;
    y[i] = sum / st;
  }
}

// x += sum_i y_i V_i on the segment's case
template <typename TV>
__global__ void __launch_bounds__(CB) k_cxupdate(CaseDev D, TV* __restrict__ x, const TV* __restrict__ V,
                                                 long vstride) {
  const int c = D.segCase[blockIdx.x];
  if (!case_on(D, c)) return;
  const double* y = D.y + (size_t)c * MAX_DIRS;
  const long e1 = 5L * D.segEnd[blockIdx.x];
  for (long e = 5L * D.segBeg[blockIdx.x] + threadIdx.x; e < e1; e += CB) {
    TV a = x[e];
    for (int i = 0; i < D.m; ++i) a += TV(y[i]) * V[(size_t)i * vstride + e];
    x[e] = a;
  }
}

// r = b - t and the case's L1 sums per equation
template <typename TV>
__global__ void __launch_bounds__(CB) k_cresid(CaseDev D, const double* __restrict__ b, const TV* __restrict__ t,
                                               TV* __restrict__ r) {
  const int c = D.segCase[blockIdx.x];
  double acc[5] = {0, 0, 0, 0, 0};
  if (case_on(D, c)) {
    const int c1 = D.segEnd[blockIdx.x];
    for (int q = D.segBeg[blockIdx.x] + threadIdx.x; q < c1; q += CB)
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const TV v = TV(b[5 * q + k]) - t[5 * q + k];
        r[5 * q + k] = v;
        acc[k] += fabs(double(v));
      }
  }
  case_finish<5>(D, c, acc, D.res + 5 * c);
}

// per case: the norm-factor sums (rho, rhoE, |rhoU|) of |A (W - avg W)| + |b|
// and |b| per equation
template <typename TV>
__global__ void __launch_bounds__(CB) k_cnormfac(CaseDev D, const double* __restrict__ b, const TV* __restrict__ t) {
  const int c = D.segCase[blockIdx.x];
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int c1 = D.segEnd[blockIdx.x];
  for (int q = D.segBeg[blockIdx.x] + threadIdx.x; q < c1; q += CB) {
    const double t0 = double(t[5 * q]), t4 = double(t[5 * q + 4]);
    const double t1 = double(t[5 * q + 1]), t2 = double(t[5 * q + 2]), t3 = double(t[5 * q + 3]);
    const double b0 = b[5 * q], b1 = b[5 * q + 1], b2 = b[5 * q + 2], b3 = b[5 * q + 3], b4 = b[5 * q + 4];
    acc[0] += fabs(t0) + fabs(b0);
    acc[1] += fabs(t4) + fabs(b4);
    acc[2] += sqrt(t1 * t1 + t2 * t2 + t3 * t3) + sqrt(b1 * b1 + b2 * b2 + b3 * b3);
    acc[3] += fabs(b0);
    acc[4] += fabs(b1);
    acc[5] += fabs(b2);
    acc[6] += fabs(b3);
    acc[7] += fabs(b4);
  }
  case_finish<8>(D, c, acc, D.nfr + 8 * c);
}

// per case: the average of W per equation (gAverage)
__global__ void __launch_bounds__(CB) k_cwavg(CaseDev D, const double* __restrict__ W) {
  const int c = D.segCase[blockIdx.x];
  double acc[5] = {0, 0, 0, 0, 0};
  const int c1 = D.segEnd[blockIdx.x];
  for (int q = D.segBeg[blockIdx.x] + threadIdx.x; q < c1; q += CB)
#pragma unroll
    for (int k = 0; k < 5; ++k) acc[k] += W[5 * q + k];
  double* avg = D.avg + 5 * c;
  if (case_finish<5>(D, c, acc, avg)) {
    const int nc = D.start[c + 1] - D.start[c];
    for (int k = 0; k < 5; ++k) avg[k] = avg[k] / nc;
  }
}

template <typename TV>
__global__ void __launch_bounds__(CB) k_cwmavg(CaseDev D, const double* __restrict__ W, TV* __restrict__ out) {
  const int c = D.segCase[blockIdx.x];
  const double* avg = D.avg + 5 * c;
  const int c1 = D.segEnd[blockIdx.x];
  for (int q = D.segBeg[blockIdx.x] + threadIdx.x; q < c1; q += CB)
#pragma unroll
    for (int k = 0; k < 5; ++k) out[5 * q + k] = TV(W[5 * q + k] - avg[k]);
}

// per case: sum of the cells' (R_rho V)^2
__global__ void __launch_bounds__(CB) k_cl2(CaseDev D, const double* __restrict__ a) {
  const int c = D.segCase[blockIdx.x];
  double acc[1] = {0.0};
  const int c1 = D.segEnd[blockIdx.x];
  for (int q = D.segBeg[blockIdx.x] + threadIdx.x; q < c1; q += CB) acc[0] += a[q];
  case_finish<1>(D, c, acc, D.l2 + c);
}

template <typename TV>
__global__ void k_cto_dW(int N, const TV* __restrict__ x, double* __restrict__ dW, int s0, int s1, int s2) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  dW[5 * c] = double(x[5 * c]);
  dW[5 * c + 1] = s0 == -1 ? 0.0 : double(x[5 * c + 1]);
  dW[5 * c + 2] = s1 == -1 ? 0.0 : double(x[5 * c + 2]);
  dW[5 * c + 3] = s2 == -1 ? 0.0 : double(x[5 * c + 3]);
  dW[5 * c + 4] = double(x[5 * c + 4]);
}

// coupledMatrix::solver::stop (coupledMatrixSolver.C:198-221) for one case
bool case_stop(const Handle& h, int nIter, const double* in, const double* fi) {
  const ics_config& c = h.cfg.c;
  if (nIter < c.min_iter) return false;
  double mx = -VGREAT, mrel = -VGREAT;
  for (int k = 0; k < 5; ++k) mx = fmax(mx, fi[k]);
  mrel = fmax(mrel, fi[0] / (in[0] + ROOTVSMALL));
  mrel = fmax(mrel, fi[4] / (in[4] + ROOTVSMALL));
  for (int k = 0; k < 3; ++k)
    if (h.m.solD[k] == 1) mrel = fmax(mrel, fi[1 + k] / (in[1 + k] + ROOTVSMALL));
  return nIter >= c.max_iter || mx < c.tolerance || mrel < c.rel_tol;
}

template <typename TV>
int gmres_cases_t(Handle& h, std::vector<int>& caseStatus) {
  CaseSet& S = h.cases;
  const int N = h.m.N, m = h.cfg.c.n_directions, n = S.n, ns = S.nseg;
  const long n5 = 5L * N;
  const long vs = (long)kstride(h);
  cudaStream_t st = h.stream;
  TV* V = (TV*)h.kv;
  TV* w = (TV*)h.kw;
  TV* x = (TV*)h.kx;
  TV* t = (TV*)h.kt;
  S.d.m = m;
  const CaseDev D = S.d;
  for (int k = 0; k < n; ++k) S.hactive[k] = S.frozen[k] ? 0 : 1;
  ICS_CUDA(cudaMemcpyAsync((void*)D.active, S.hactive, n * sizeof(int), cudaMemcpyHostToDevice, st));
  ICS_CUDA(cudaMemsetAsync(D.status, 0, n * sizeof(int), st));
  ICS_CUDA(cudaMemsetAsync(&h.ks->status, 0, sizeof(int), st));  // bounded waits of the sync-free sweeps
  // norm factors and initial residuals per case (gmres.C:812-850)
  ICS_LAUNCH(h, ICS_K_VECTOR, k_cwavg<<<ns, CB, 0, st>>>(D, h.W));
  ICS_LAUNCH(h, ICS_K_VECTOR, k_cwmavg<TV><<<ns, CB, 0, st>>>(D, h.W, w));
  spmv(h, w, t);
  ICS_LAUNCH(h, ICS_K_VECTOR, k_cnormfac<TV><<<ns, CB, 0, st>>>(D, h.src, t));
  ICS_CUDA(cudaMemcpyAsync(S.hnfr, D.nfr, 8ull * n * sizeof(double), cudaMemcpyDeviceToHost, st));
  ICS_CUDA(cudaStreamSynchronize(st));
  std::vector<double> nf(3 * n), fin(S.initRes);
  for (int k = 0; k < n; ++k) {
    const double* q = S.hnfr + 8 * k;
    for (int j = 0; j < 3; ++j) nf[3 * k + j] = q[j] + VSMALL;
    double* in = &S.initRes[5 * k];
    if (!S.hactive[k]) continue;
    in[0] = q[3] / nf[3 * k];
    in[1] = q[4] / nf[3 * k + 2];
    in[2] = q[5] / nf[3 * k + 2];
    in[3] = q[6] / nf[3 * k + 2];
    in[4] = q[7] / nf[3 * k + 1];
    std::copy(in, in + 5, &fin[5 * k]);
  }
  std::vector<int> nIter(n, 0);
  caseStatus.assign(n, ICS_OK);
  ICS_CUDA(cudaMemsetAsync(x, 0, n5 * sizeof(TV), st));
  to_vec(h, h.src, w);
  auto cycle = [&]() {
    precondition(h, w);
    ICS_LAUNCH(h, ICS_K_MGS, k_cmgs<TV><<<ns, CB, 0, st>>>(D, w, nullptr, 0, nullptr, 0, 0, 1, 0));
    // with the fused operator (each row scaled by its own case's norm) the
    // unnormalised vector alternates between w and t, as in the single-system
    // cycle; the cycle's residual goes back to w
    TV* wb[2] = {w, t};
    for (int i = 0; i < m; ++i) {
      TV* vi = V + (size_t)i * vs;
      TV* wc = w;
      if (fused_operator(h, wb[i & 1], wb[(i + 1) & 1], vi)) {
        wc = wb[(i + 1) & 1];
      } else {
        ICS_LAUNCH(h, ICS_K_VECTOR, k_cscale<TV><<<ns, CB, 0, st>>>(D, w, vi));
        spmv(h, vi, w);
        precondition(h, w);
      }
      for (int j = 0; j <= i; ++j) {
        const TV* vprev = j > 0 ? V + (size_t)(j - 1) * vs : nullptr;
        ICS_LAUNCH(h, ICS_K_MGS, k_cmgs<TV><<<ns, CB, 0, st>>>(D, wc, vprev, (j - 1) * m + i, V + (size_t)j * vs,
                                                               j * m + i, -1, 0, i));
      }
      ICS_LAUNCH(h, ICS_K_MGS, k_cmgs<TV><<<ns, CB, 0, st>>>(D, wc, vi, i * m + i, nullptr, 0, 1, 2, i));
    }
    ICS_LAUNCH(h, ICS_K_SCALAR, k_cbacksub<<<(n + 63) / 64, 64, 0, st>>>(D));
    ICS_LAUNCH(h, ICS_K_VECTOR, k_cxupdate<TV><<<ns, CB, 0, st>>>(D, x, V, vs));
    spmv(h, x, t);
    ICS_LAUNCH(h, ICS_K_VECTOR, k_cresid<TV><<<ns, CB, 0, st>>>(D, h.src, t, w));
  };
  // the captured launches hold DevMesh and CaseDev by value
  const int key = 30000000 + (h.m.vjslot ? 10000000 : 0) + h.cfg.c.preconditioner * 100000 + prec(h) * 1000 + m;
  const bool useGraph = !h.prof;
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
    h.launches = before;
    h.cycleKey = key;
  }
  int status = ICS_OK;
  for (bool any = true; any;) {
    if (useGraph) {
      ICS_CUDA(cudaGraphLaunch(h.cycleExec, st));
      h.launches += h.cycleLaunches;
    } else {
      cycle();
    }
    ICS_CUDA(cudaGetLastError());
    int sweepStatus = 0;
    ICS_CUDA(cudaMemcpyAsync(S.hres, D.res, 5ull * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaMemcpyAsync(S.hstatus, D.status, n * sizeof(int), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaMemcpyAsync(&sweepStatus, &h.ks->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaStreamSynchronize(st));
    if (sweepStatus & 8) {
      status = ICS_ERR_TIMEOUT;
      break;
    }
    any = false;
    for (int k = 0; k < n; ++k) {
      if (!S.hactive[k]) continue;
      nIter[k]++;
      if (S.hstatus[k]) {
        caseStatus[k] = (S.hstatus[k] & 4) ? ICS_ERR_NONFINITE : ICS_ERR_BREAKDOWN;
        S.hactive[k] = 0;
        continue;
      }
      const double* rs = S.hres + 5 * k;
      double* fi = &fin[5 * k];
      bool finite = true;
      fi[0] = rs[0] / nf[3 * k];
      fi[4] = rs[4] / nf[3 * k + 1];
      for (int j = 0; j < 3; ++j) fi[1 + j] = h.m.solD[j] == -1 ? 0.0 : rs[1 + j] / nf[3 * k + 2];
      for (int j = 0; j < 5; ++j) finite = finite && std::isfinite(fi[j]);
      if (!finite) {
        caseStatus[k] = ICS_ERR_NONFINITE;
        S.hactive[k] = 0;
        continue;
      }
      if (case_stop(h, nIter[k], &S.initRes[5 * k], fi))
        S.hactive[k] = 0;
      else
        any = true;
    }
    if (any)
      ICS_CUDA(cudaMemcpyAsync((void*)D.active, S.hactive, n * sizeof(int), cudaMemcpyHostToDevice, st));
  }
  ICS_LAUNCH(h, ICS_K_VECTOR, k_cto_dW<TV><<<grid_for(N, 256), 256, 0, st>>>(N, x, h.dW, h.m.solD[0], h.m.solD[1],
                                                                             h.m.solD[2]));
  ICS_CUDA(cudaStreamSynchronize(st));
  for (int k = 0; k < n; ++k) {
    S.cycles[k] = S.frozen[k] ? 0 : nIter[k];
    if (!S.frozen[k]) std::copy(&fin[5 * k], &fin[5 * k] + 5, &S.finRes[5 * k]);
  }
  return status;
}

// the next 256-byte aligned array of count T at offset off of base
template <typename T>
T* carve(char* base, size_t& off, size_t count) {
  T* r = base ? reinterpret_cast<T*>(base + off) : nullptr;
  off += ((count * sizeof(T) + 255) / 256) * 256;
  return r;
}

}  // namespace

void free_cases(Handle& h) {
  CaseSet& S = h.cases;
  if (S.mem) cudaFree(S.mem);
  if (S.hres) cudaFreeHost(S.hres);
  S = CaseSet();
  h.m.caseOf = nullptr;
  h.m.caseSer = nullptr;
  h.m.caseBeta = nullptr;
  h.m.caseActive = nullptr;
  h.m.caseStatus = nullptr;
}

void set_cases(Handle& h, int n, const int* start) {
  const int N = h.m.N;
  if (n < 1 || !start || start[0] != 0 || start[n] != N) throw std::string("case_start must run from 0 to n_cells");
  for (int k = 0; k < n; ++k)
    if (start[k + 1] <= start[k]) throw std::string("case_start must be strictly increasing");
  if (h.m.nInst > 1) throw std::string("stacked cases are not combined with Harmonic Balance");
  if (h.m.ncyc > 0) throw std::string("stacked cases carry no cyclic patches");
  if (h.cfg.c.solver != ICS_SOLVER_GMRES) throw std::string("stacked cases need the GMRES solver");
  if (h.scalarOn) throw std::string("stacked cases carry no passive scalar");
  std::vector<int> caseOf(N);
  for (int k = 0; k < n; ++k)
    for (int c = start[k]; c < start[k + 1]; ++c) caseOf[c] = k;
  if (h.m.F) {
    std::vector<int> own(h.m.F), nei(h.m.F);
    ICS_CUDA(cudaMemcpy(own.data(), h.m.own, h.m.F * sizeof(int), cudaMemcpyDeviceToHost));
    ICS_CUDA(cudaMemcpy(nei.data(), h.m.nei, h.m.F * sizeof(int), cudaMemcpyDeviceToHost));
    for (int f = 0; f < h.m.F; ++f)
      if (caseOf[own[f]] != caseOf[nei[f]]) throw std::string("an internal face joins two cases");
  }
  std::vector<int> segCase, segBeg, segEnd, caseSeg(n + 1);
  for (int k = 0; k < n; ++k) {
    caseSeg[k] = (int)segCase.size();
    for (int b = start[k]; b < start[k + 1]; b += SEG_CELLS) {
      segCase.push_back(k);
      segBeg.push_back(b);
      segEnd.push_back(std::min(b + SEG_CELLS, start[k + 1]));
    }
  }
  const int ns = (int)segCase.size();
  caseSeg[n] = ns;
  free_cases(h);
  drop_graphs(h);
  CaseSet& S = h.cases;
  CaseDev& D = S.d;
  D.n = n;
  D.m = h.cfg.c.n_directions;
  int *dSegCase, *dSegBeg, *dSegEnd, *dCaseSeg, *dStart;
  // one allocation, laid out twice: for its size, then over the allocation
  auto layout = [&](char* base) {
    size_t off = 0;
    dSegCase = carve<int>(base, off, ns);
    dSegBeg = carve<int>(base, off, ns);
    dSegEnd = carve<int>(base, off, ns);
    dCaseSeg = carve<int>(base, off, n + 1);
    dStart = carve<int>(base, off, n + 1);
    D.active = carve<int>(base, off, n);
    D.status = carve<int>(base, off, n);
    S.caseOf = carve<int>(base, off, N);
    D.counter = carve<unsigned int>(base, off, n);
    D.partials = carve<double>(base, off, (size_t)PSTRIDE * ns);
    D.H = carve<double>(base, off, (size_t)n * HSTRIDE);
    D.c = carve<double>(base, off, (size_t)n * MAX_DIRS);
    D.s = carve<double>(base, off, (size_t)n * MAX_DIRS);
    D.y = carve<double>(base, off, (size_t)n * MAX_DIRS);
    D.bh = carve<double>(base, off, (size_t)n * (MAX_DIRS + 1));
    D.beta = carve<double>(base, off, n);
    D.red = carve<double>(base, off, 2ull * n);
    D.res = carve<double>(base, off, 5ull * n);
    D.nfr = carve<double>(base, off, 8ull * n);
    D.avg = carve<double>(base, off, 5ull * n);
    D.l2 = carve<double>(base, off, n);
    S.ser = carve<double>(base, off, n);
    return off;
  };
  const size_t bytes = layout(nullptr);
  ICS_CUDA(cudaMalloc(&S.mem, bytes));
  ICS_CUDA(cudaMemset(S.mem, 0, bytes));
  layout((char*)S.mem);
  ICS_CUDA(cudaMemcpy(dSegCase, segCase.data(), ns * sizeof(int), cudaMemcpyHostToDevice));
  ICS_CUDA(cudaMemcpy(dSegBeg, segBeg.data(), ns * sizeof(int), cudaMemcpyHostToDevice));
  ICS_CUDA(cudaMemcpy(dSegEnd, segEnd.data(), ns * sizeof(int), cudaMemcpyHostToDevice));
  ICS_CUDA(cudaMemcpy(dCaseSeg, caseSeg.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
  ICS_CUDA(cudaMemcpy(dStart, start, (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
  ICS_CUDA(cudaMemcpy(S.caseOf, caseOf.data(), N * sizeof(int), cudaMemcpyHostToDevice));
  D.segCase = dSegCase;
  D.segBeg = dSegBeg;
  D.segEnd = dSegEnd;
  D.caseSeg = dCaseSeg;
  D.start = dStart;
  // pinned mirrors: res [5n], nfr [8n], l2 [n], ser [n], status [n], active [n]
  ICS_CUDA(cudaMallocHost(&S.hres, sizeof(double) * 15ull * n + sizeof(int) * 2ull * n));
  S.hnfr = S.hres + 5 * n;
  S.hl2 = S.hnfr + 8 * n;
  S.hser = S.hl2 + n;
  S.hstatus = reinterpret_cast<int*>(S.hser + n);
  S.hactive = S.hstatus + n;
  S.n = n;
  S.nseg = ns;
  S.start.assign(start, start + n + 1);
  S.ctl.assign(n, PseudoControl());
  S.initRes.assign(5 * n, 0.0);
  S.prevRes.assign(5 * n, 0.0);
  S.finRes.assign(5 * n, 0.0);
  S.initValid.assign(n, 0);
  S.prevValid.assign(n, 0);
  S.frozen.assign(n, 0);
  S.cycles.assign(n, 0);
  h.m.caseOf = S.caseOf;
  h.m.caseSer = S.ser;
  h.m.caseBeta = D.beta;
  h.m.caseActive = D.active;
  h.m.caseStatus = D.status;
}

int gmres_cases(Handle& h, std::vector<int>& caseStatus) {
  return prec(h) == ICS_PREC_MIXED ? gmres_cases_t<float>(h, caseStatus) : gmres_cases_t<double>(h, caseStatus);
}

// per-case sums of (R_rho V)^2 from the last residual into the host mirror
void case_l2(Handle& h) {
  CaseSet& S = h.cases;
  ICS_LAUNCH(h, ICS_K_VECTOR, k_cl2<<<S.nseg, CB, 0, h.stream>>>(S.d, h.scratch));
  ICS_CUDA(cudaMemcpyAsync(S.hl2, S.d.l2, S.n * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
  ICS_CUDA(cudaStreamSynchronize(h.stream));
}

// the cases' SER factors of the next residual (host mirror -> device)
void case_upload_ser(Handle& h) {
  CaseSet& S = h.cases;
  ICS_CUDA(cudaMemcpyAsync(S.ser, S.hser, S.n * sizeof(double), cudaMemcpyHostToDevice, h.stream));
}

}  // namespace ics
