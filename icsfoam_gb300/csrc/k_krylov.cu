// Matrix-free Krylov solves with the exact derivative of the residual:
//
// with A = s V / dtau - d(R V)/dW (s = 0 or 1: the steady operator, or the
// pseudo-time step's; the reference's Jacobian approximates A with s = 1):
//
//   adjoint  A^T psi = g             operator: the reverse-mode product
//                                    (launch_residual_vjp, no stored Jacobian)
//   tangent  A x = b                 operator: the forward-mode product
//                                    (launch_residual_tangent): a matrix-free
//                                    Newton-Krylov step
//
// Restarted GMRES with right preconditioning (so the Arnoldi residual is the
// true residual of the unpreconditioned system) and classical Gram-Schmidt
// applied twice (CGS2: one fused multi-dot pass over the basis and one update
// pass per sweep, stable for an FP32 basis).  The operator and the
// preconditioner act on FP64 vectors; the Krylov basis is FP64 or FP32
// (ICS_PREC_MIXED), its dot products accumulate in FP64.  The preconditioner
// is the LU-SGS of the reference's approximate Jacobian (ics_assemble_jacobian,
// lusgs.C): for the tangent system as assembled, for the adjoint system
// transposed -- M^T = (D + U^T) D^-1 (D + L^T) is the LU-SGS of A^T, whose
// sliced-ELL rows hold the transposed blocks of the mirror slots (same
// structure, same level schedule, same scalar diagonal).  The Hessenberg
// matrix, Givens rotations and the small triangular solve live on the host;
// every dot product is a deterministic two-stage device reduction.
#include <cmath>
#include <functional>
#include <vector>

#include "ics_internal.cuh"

namespace ics {

// LU-SGS sweeps of k_linalg.cu on an FP64 vector with given slot storage
void lusgs_with(Handle& h, const void* blk, const void* rD, bool fp32, double* r);

namespace {

constexpr int KB = 256;          // threads per reduction block
constexpr int KBLOCKS = 1216;    // 8 x 152 SMs

// ----------------------------------------------- transposed approximate Jacobian
// mirror[slot*32 + lane] = position (slot'*32 + lane') of the same face in the
// row of the column cell
__global__ void k_mirror(DevMesh m, int* __restrict__ mirror) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int s = c >> 5, lane = c & 31, base = m.slot_base[s];
  for (int t = 0; t < m.nslot[c]; ++t) {
    const int pos = (base + t) * 32 + lane;
    const int col = m.scol[pos];
    const int code = m.sface[pos];
    const int f = code >= 0 ? code : ~code;
    const int s2 = col >> 5, l2 = col & 31, b2 = m.slot_base[s2];
    int found = -1;
    for (int t2 = 0; t2 < m.nslot[col]; ++t2) {
      const int p2 = (b2 + t2) * 32 + l2;
      const int c2 = m.sface[p2];
      if ((c2 >= 0 ? c2 : ~c2) == f) {
        found = p2;
        break;
      }
    }
    mirror[pos] = found;
  }
}

// blkT slot (row c, column n) = (slot (row n, column c))^T, 25 FP64 entries
// from the expanded slots ex [nslots][25][32]
__global__ void k_transpose_slots(DevMesh m, const int* __restrict__ mirror, const double* __restrict__ ex,
                                  double* __restrict__ blkT) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int s = c >> 5, lane = c & 31, base = m.slot_base[s];
  for (int t = 0; t < m.nslot[c]; ++t) {
    const int pos = (base + t) * 32 + lane;
    const int mp = mirror[pos];
    const size_t ms = mp >> 5, ml = mp & 31;
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j)
        blkT[((size_t)(base + t) * 25 + 5 * i + j) * 32 + lane] = mp >= 0 ? ex[(ms * 25 + 5 * j + i) * 32 + ml] : 0.0;
  }
}

template <typename TS>
__global__ void k_to_fp64(long n, const TS* __restrict__ a, double* __restrict__ b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    b[i] = double(a[i]);
}
template <typename TD>
__global__ void k_from_fp64(long n, const double* __restrict__ a, TD* __restrict__ b, double s) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    b[i] = TD(a[i] * s);
}

// ------------------------------------------------------------- reductions
// partials[blk][j] = sum over the block's elements of w . V_j, j < k
template <typename TW, typename TV>
__global__ void __launch_bounds__(KB) k_mdot(long n, const TW* __restrict__ w, const TV* __restrict__ V, long stride,
                                             int k, double* __restrict__ partials) {
  __shared__ double sm[KB / 32];
  const int ln = threadIdx.x & 31, wp = threadIdx.x >> 5;
  for (int j = 0; j < k; ++j) {
    const TV* v = V + (size_t)j * stride;
    double a = 0.0;
    for (long i = blockIdx.x * (long)KB + threadIdx.x; i < n; i += (long)gridDim.x * KB)
      a += double(w[i]) * double(v[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (ln == 0) sm[wp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int q = 0; q < KB / 32; ++q) t += sm[q];
      partials[(size_t)blockIdx.x * k + j] = t;
    }
    __syncthreads();
  }
}

// out[j] = sum over blocks, in block order
__global__ void k_fold(const double* __restrict__ partials, int nblk, int k, double* __restrict__ out) {
  const int j = threadIdx.x;
  if (j >= k) return;
  double t = 0.0;
  for (int b = 0; b < nblk; ++b) t += partials[(size_t)b * k + j];
  out[j] = t;
}

// w -= sum_j coef_j V_j
template <typename TV>
__global__ void k_subtract(long n, TV* __restrict__ w, const TV* __restrict__ V, long stride, int k,
                           const double* __restrict__ coef) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double a = double(w[i]);
    for (int j = 0; j < k; ++j) a -= coef[j] * double(V[(size_t)j * stride + i]);
    w[i] = TV(a);
  }
}

// u = sum_j y_j V_j (FP64)
template <typename TV>
__global__ void k_combine(long n, double* __restrict__ u, const TV* __restrict__ V, long stride, int k,
                          const double* __restrict__ y) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double a = 0.0;
    for (int j = 0; j < k; ++j) a += y[j] * double(V[(size_t)j * stride + i]);
    u[i] = a;
  }
}

__global__ void k_axpy64(long n, double* __restrict__ x, const double* __restrict__ u, double a) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    x[i] += a * u[i];
}

// out = s (V rPDT) in - out: the operator s V / dtau - d(R V)/dW from the product in out
__global__ void k_shift(int N, double s, const double* __restrict__ rPDT, const double* __restrict__ V,
                        const double* __restrict__ in, double* __restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < 5L * N; i += (long)gridDim.x * blockDim.x) {
    const long c = i / 5;
    out[i] = s * rPDT[c] * V[c] * in[i] - out[i];
  }
}

// r = b - t
__global__ void k_sub64(long n, const double* __restrict__ b, const double* __restrict__ t, double* __restrict__ r) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    r[i] = b[i] - t[i];
}

struct Workspace {
  std::vector<void*> ptrs;
  void* get(size_t bytes) {
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) throw CudaError(e, "cudaMalloc", __FILE__, __LINE__);
    ptrs.push_back(p);
    return p;
  }
  ~Workspace() {
    for (void* p : ptrs) cudaFree(p);
  }
};

struct Ops {
  std::function<void(const double*, double*)> op;  // out = A in (device FP64 [5N])
  std::function<void(double*)> pc;                 // r <- M^-1 r in place (may be empty)
};

template <typename TV>
int gmres_matfree(Handle& h, const Ops& A, const double* b, double* x, const ics_krylov_opts& o,
                  ics_krylov_result* res) {
  const long n = 5L * h.m.N;
  const int m = o.n_directions;
  const long stride = ((n + 63) / 64) * 64;
  cudaStream_t st = h.stream;
  Workspace ws;
  TV* V = (TV*)ws.get((size_t)(m + 1) * stride * sizeof(TV));
  double* d1 = (double*)ws.get(n * sizeof(double));
  double* d2 = (double*)ws.get(n * sizeof(double));
  double* partials = (double*)ws.get((size_t)KBLOCKS * (m + 1) * sizeof(double));
  double* dv = (double*)ws.get((m + 2) * sizeof(double));
  const int G = KBLOCKS;
  // <a, V_0..V_{k-1}> to the host
  auto mdot = [&](const auto* a, const TV* Vb, int k, double* out) {
    using TA = std::remove_cv_t<std::remove_pointer_t<decltype(a)>>;
    ICS_LAUNCH(h, ICS_K_MGS, (k_mdot<TA, TV><<<G, KB, 0, st>>>(n, a, Vb, stride, k, partials)));
    ICS_LAUNCH(h, ICS_K_MGS, k_fold<<<1, 64, 0, st>>>(partials, G, k, dv));
    ICS_CUDA(cudaMemcpyAsync(out, dv, k * sizeof(double), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaStreamSynchronize(st));
  };
  auto norm64 = [&](const double* a) {
    double s = 0.0;
    ICS_LAUNCH(h, ICS_K_MGS, (k_mdot<double, double><<<G, KB, 0, st>>>(n, a, a, 0, 1, partials)));
    ICS_LAUNCH(h, ICS_K_MGS, k_fold<<<1, 64, 0, st>>>(partials, G, 1, dv));
    ICS_CUDA(cudaMemcpyAsync(&s, dv, sizeof(double), cudaMemcpyDeviceToHost, st));
    ICS_CUDA(cudaStreamSynchronize(st));
    return std::sqrt(s);
  };
  ICS_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), st));
  const double bnorm = norm64(b);
  res->iterations = res->cycles = 0;
  res->rel_residual = 0.0;
  res->converged = 1;
  if (bnorm == 0.0) return ICS_OK;
  // r0 = b (x0 = 0)
  ICS_CUDA(cudaMemcpyAsync(d1, b, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  double beta = bnorm;
  std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), y(m), hv(m + 1), h2(m + 1);
  res->converged = 0;
  while (res->cycles < o.max_cycles) {
    ICS_LAUNCH(h, ICS_K_VECTOR, (k_from_fp64<TV><<<G, KB, 0, st>>>(n, d1, V, 1.0 / beta)));
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    bool done = false;
    for (int i = 0; i < m; ++i) {
      // w = A M^-1 v_i, into V_{i+1}
      TV* vi = V + (size_t)i * stride;
      TV* w = V + (size_t)(i + 1) * stride;
      ICS_LAUNCH(h, ICS_K_VECTOR, (k_to_fp64<TV><<<G, KB, 0, st>>>(n, vi, d1)));
      if (A.pc) A.pc(d1);
      A.op(d1, d2);
      ICS_LAUNCH(h, ICS_K_VECTOR, (k_from_fp64<TV><<<G, KB, 0, st>>>(n, d2, w, 1.0)));
      // CGS2 against V_0..V_i
      mdot(w, V, i + 1, hv.data());
      ICS_CUDA(cudaMemcpyAsync(dv, hv.data(), (i + 1) * sizeof(double), cudaMemcpyHostToDevice, st));
      ICS_LAUNCH(h, ICS_K_MGS, (k_subtract<TV><<<G, KB, 0, st>>>(n, w, V, stride, i + 1, dv)));
      mdot(w, V, i + 1, h2.data());
      ICS_CUDA(cudaMemcpyAsync(dv, h2.data(), (i + 1) * sizeof(double), cudaMemcpyHostToDevice, st));
      ICS_LAUNCH(h, ICS_K_MGS, (k_subtract<TV><<<G, KB, 0, st>>>(n, w, V, stride, i + 1, dv)));
      double hn2 = 0.0;
      mdot(w, w, 1, &hn2);
      const double hn = std::sqrt(hn2);
      for (int j = 0; j <= i; ++j) H[j * m + i] = hv[j] + h2[j];
      H[(i + 1) * m + i] = hn;
      if (hn > 0.0) {
        ICS_LAUNCH(h, ICS_K_VECTOR, (k_to_fp64<TV><<<G, KB, 0, st>>>(n, w, d2)));
        ICS_LAUNCH(h, ICS_K_VECTOR, (k_from_fp64<TV><<<G, KB, 0, st>>>(n, d2, w, 1.0 / hn)));
      }
      // Givens rotations of the new column
      for (int j = 0; j < i; ++j) {
        const double a = H[j * m + i], c2 = H[(j + 1) * m + i];
        H[j * m + i] = cs[j] * a + sn[j] * c2;
        H[(j + 1) * m + i] = -sn[j] * a + cs[j] * c2;
      }
      const double a = H[i * m + i], c2 = H[(i + 1) * m + i];
      const double r = std::hypot(a, c2);
      cs[i] = r > 0 ? a / r : 1.0;
      sn[i] = r > 0 ? c2 / r : 0.0;
      H[i * m + i] = r;
      H[(i + 1) * m + i] = 0.0;
      g[i + 1] = -sn[i] * g[i];
      g[i] = cs[i] * g[i];
      k = i + 1;
      res->iterations++;
      if (std::fabs(g[i + 1]) <= o.rel_tol * bnorm || hn == 0.0) {
        done = true;
        break;
      }
    }
    // y = H^-1 g, u = M^-1 V y, x += u
    for (int i = k - 1; i >= 0; --i) {
      double s = g[i];
      for (int j = i + 1; j < k; ++j) s -= H[i * m + j] * y[j];
      y[i] = H[i * m + i] != 0.0 ? s / H[i * m + i] : 0.0;
    }
    ICS_CUDA(cudaMemcpyAsync(dv, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, st));
    ICS_LAUNCH(h, ICS_K_VECTOR, (k_combine<TV><<<G, KB, 0, st>>>(n, d2, V, stride, k, dv)));
    if (A.pc) A.pc(d2);
    ICS_LAUNCH(h, ICS_K_VECTOR, k_axpy64<<<G, KB, 0, st>>>(n, x, d2, 1.0));
    res->cycles++;
    // true residual r = b - A x
    A.op(x, d2);
    ICS_LAUNCH(h, ICS_K_VECTOR, k_sub64<<<G, KB, 0, st>>>(n, b, d2, d1));
    beta = norm64(d1);
    res->rel_residual = beta / bnorm;
    if (!std::isfinite(beta)) return ICS_ERR_NONFINITE;
    if (beta <= o.rel_tol * bnorm) {
      res->converged = 1;
      break;
    }
    if (done && beta == 0.0) break;
  }
  ICS_CUDA(cudaGetLastError());
  return ICS_OK;
}

}  // namespace

// transposed slots and FP64 scalar diagonal of the assembled approximate
// Jacobian (for the adjoint's LU-SGS); owned by the workspace of one solve
struct TransposedJacobian {
  double* blkT = nullptr;
  double* rD = nullptr;
};

static TransposedJacobian transpose_jacobian(Handle& h, Workspace& ws) {
  const size_t slots = (size_t)h.m.nslots;
  TransposedJacobian t;
  double* ex = (double*)ws.get(slots * 25 * 32 * sizeof(double));
  int* mirror = (int*)ws.get(slots * 32 * sizeof(int));
  t.blkT = (double*)ws.get(slots * 25 * 32 * sizeof(double));
  t.rD = (double*)ws.get((size_t)h.m.N * sizeof(double));
  launch_expand_slots(h, ex);
  const int N = h.m.N;
  ICS_LAUNCH(h, ICS_K_VECTOR, k_mirror<<<grid_for(N, 128), 128, 0, h.stream>>>(h.m, mirror));
  ICS_LAUNCH(h, ICS_K_VECTOR, k_transpose_slots<<<grid_for(N, 128), 128, 0, h.stream>>>(h.m, mirror, ex, t.blkT));
  if (h.jacPrecision == ICS_PREC_MIXED)
    ICS_LAUNCH(h, ICS_K_VECTOR, (k_to_fp64<float><<<KBLOCKS, KB, 0, h.stream>>>(N, (const float*)h.rD, t.rD)));
  else
    ICS_CUDA(cudaMemcpyAsync(t.rD, h.rD, N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
  ICS_CUDA(cudaGetLastError());
  return t;
}

static void check_opts(const Handle& h, const ics_krylov_opts& o) {
  if (o.n_directions < 1 || o.n_directions > 64 || o.max_cycles < 1 || !(o.rel_tol > 0.0) ||
      (o.precision != ICS_PREC_FP64 && o.precision != ICS_PREC_MIXED) ||
      (o.preconditioner != ICS_PC_NONE && o.preconditioner != ICS_PC_LUSGS) ||
      (o.pseudo_time != 0 && o.pseudo_time != 1))
    throw std::string("krylov options: n_directions in [1, 64], max_cycles >= 1, rel_tol > 0, "
                      "precision FP64/MIXED, preconditioner NONE/LUSGS, pseudo_time 0/1");
  if (o.preconditioner == ICS_PC_LUSGS && !h.haveMatrix)
    throw std::string("the LU-SGS preconditioner needs ics_assemble_jacobian at this state");
  if (h.m.ncyc > 0 && o.preconditioner == ICS_PC_LUSGS)
    throw std::string("the LU-SGS preconditioner of the Krylov solves does not carry cyclic couplings");
}

int adjoint_solve(Handle& h, const double* g, double* psi, const ics_krylov_opts& o, ics_krylov_result* res) {
  check_opts(h, o);
  const std::string why = residual_vjp_unsupported(h);
  if (!why.empty()) throw why;
  Workspace ws;
  Ops A;
  const double sh = o.pseudo_time ? 1.0 : 0.0;
  A.op = [&](const double* in, double* out) {
    launch_residual_vjp(h, in, out);
    ICS_LAUNCH(h, ICS_K_VECTOR, k_shift<<<KBLOCKS, KB, 0, h.stream>>>(h.m.N, sh, h.rPDT, h.m.V, in, out));
  };
  TransposedJacobian T;
  if (o.preconditioner == ICS_PC_LUSGS) {
    T = transpose_jacobian(h, ws);
    A.pc = [&](double* r) {
      // the non-LF viscous slot parts are not part of the transposed blocks
      const void* vs = h.m.vjslot;
      h.m.vjslot = nullptr;
      lusgs_with(h, T.blkT, T.rD, false, r);
      h.m.vjslot = vs;
    };
  }
  return o.precision == ICS_PREC_MIXED ? gmres_matfree<float>(h, A, g, psi, o, res)
                                       : gmres_matfree<double>(h, A, g, psi, o, res);
}

int tangent_solve(Handle& h, const double* b, double* x, const ics_krylov_opts& o, ics_krylov_result* res) {
  check_opts(h, o);
  Ops A;
  const double sh = o.pseudo_time ? 1.0 : 0.0;
  A.op = [&](const double* in, double* out) {
    launch_residual_tangent(h, in, out);
    ICS_LAUNCH(h, ICS_K_VECTOR, k_shift<<<KBLOCKS, KB, 0, h.stream>>>(h.m.N, sh, h.rPDT, h.m.V, in, out));
  };
  if (o.preconditioner == ICS_PC_LUSGS)
    A.pc = [&](double* r) { lusgs_with(h, h.blk, h.rD, h.jacPrecision == ICS_PREC_MIXED, r); };
  return o.precision == ICS_PREC_MIXED ? gmres_matfree<float>(h, A, b, x, o, res)
                                       : gmres_matfree<double>(h, A, b, x, o, res);
}

// ----------------------------------------------------- pressure force
// J = sum over the patch's faces of p (S . dir), with p the face's cell
// pressure (the patch's pressure is zeroGradient), and dJ/dW per cell:
// p = (R / Cv) (rhoE - |rhoU|^2 / (2 rho))
__global__ void k_pressure_force(DevMesh m, int patch, double d0, double d1, double d2, double RbyCv,
                                 const double* __restrict__ W, const double* __restrict__ prim,
                                 double* __restrict__ jc, double* __restrict__ dJ) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.N) return;
  const int B = m.B;
  double s = 0.0;
  for (int e = m.bptr[c]; e < m.bptr[c + 1]; ++e) {
    const int b = m.bface[e];
    if (m.bpatch[b] != patch) continue;
    s += m.bSf[b] * d0 + m.bSf[B + b] * d1 + m.bSf[2 * B + b] * d2;
  }
  jc[c] = prim[c] * s;
  if (dJ) {
    const double rho = W[5 * c];
    const double U[3] = {W[5 * c + 1] / rho, W[5 * c + 2] / rho, W[5 * c + 3] / rho};
    dJ[5 * c] = s * RbyCv * 0.5 * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
    dJ[5 * c + 1] = -s * RbyCv * U[0];
    dJ[5 * c + 2] = -s * RbyCv * U[1];
    dJ[5 * c + 3] = -s * RbyCv * U[2];
    dJ[5 * c + 4] = s * RbyCv;
  }
}

double device_sum(Handle& h, const double* a, int n);

double pressure_force(Handle& h, int patch, const double dir[3], double* dJdW_dev) {
  const int N = h.m.N;
  Workspace ws;
  double* jc = (double*)ws.get((size_t)N * sizeof(double));
  ICS_LAUNCH(h, ICS_K_VECTOR, k_pressure_force<<<grid_for(N, 128), 128, 0, h.stream>>>(
                                  h.m, patch, dir[0], dir[1], dir[2], h.cfg.c.R / h.cfg.Cv, h.W, h.prim, jc,
                                  dJdW_dev));
  return device_sum(h, jc, N);
}

}  // namespace ics
