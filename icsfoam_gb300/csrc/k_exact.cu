// Exact (fully differentiated) Jacobian of the residual source and its
// transpose product.
//
// The residual of a cell depends on the states within two face hops (the
// limited gradients of its neighbours enter its face reconstructions; the
// viscous face gradients likewise), plus, for Harmonic Balance, the same cell
// of the other instances.  That stencil is built once on the host; the cells
// are coloured so that no two cells of one colour influence a common
// residual, and every (colour, component) pair costs one forward-mode
// Jacobian-vector product whose result lands, row by row, in the block of
// the unique seeded cell of the row's stencil (Curtis-Powell-Reid
// compression).  The transpose product J^T u is then a gather over the same
// structurally symmetric stencil.
//
// Blocks are row-major [i][k] = d(source_i of the row cell)/d(W_k of the
// column cell), stored [nnz][25] with the row's columns in increasing order.
#include <algorithm>
#include <vector>

#include "dual.cuh"
#include "ics_internal.cuh"

namespace ics {

__global__ void k_seed_colour(int N, const int* __restrict__ colour, int cid, int comp, double* __restrict__ v) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const double one = colour[c] == cid ? 1.0 : 0.0;
#pragma unroll
  for (int k = 0; k < 5; ++k) v[5 * c + k] = k == comp ? one : 0.0;
}

__global__ void k_exact_scatter(int N, const int* __restrict__ ptr, const int* __restrict__ col,
                                const int* __restrict__ colour, int cid, int comp, const double* __restrict__ jv,
                                double* __restrict__ blk) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N) return;
  for (int j = ptr[r]; j < ptr[r + 1]; ++j) {
    if (colour[col[j]] != cid) continue;
#pragma unroll
    for (int i = 0; i < 5; ++i) blk[(size_t)j * 25 + 5 * i + comp] = jv[5 * r + i];
  }
}

// y_c = sum over the rows r of c's stencil of J(r, c)^T u_r
__global__ void k_exact_vjp(int N, const int* __restrict__ ptr, const int* __restrict__ col,
                            const int* __restrict__ tpos, const double* __restrict__ blk,
                            const double* __restrict__ u, double* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  double acc[5] = {0, 0, 0, 0, 0};
  for (int j = ptr[c]; j < ptr[c + 1]; ++j) {
    const int r = col[j];
    const double* b = blk + (size_t)tpos[j] * 25;
    double ur[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) ur[i] = u[5 * r + i];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      double s = 0;
#pragma unroll
      for (int i = 0; i < 5; ++i) s += b[5 * i + k] * ur[i];
      acc[k] += s;
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) y[5 * c + k] = acc[k];
}

// y_r = sum over the stencil of r of J(r, c) x_c
__global__ void k_exact_jvp(int N, const int* __restrict__ ptr, const int* __restrict__ col,
                            const double* __restrict__ blk, const double* __restrict__ x, double* __restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N) return;
  double acc[5] = {0, 0, 0, 0, 0};
  for (int j = ptr[r]; j < ptr[r + 1]; ++j) {
    const int c = col[j];
    const double* b = blk + (size_t)j * 25;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      double s = 0;
#pragma unroll
      for (int k = 0; k < 5; ++k) s += b[5 * i + k] * x[5 * c + k];
      acc[i] += s;
    }
  }
#pragma unroll
  for (int i = 0; i < 5; ++i) y[5 * r + i] = acc[i];
}

namespace {

template <typename T>
T* xalloc(size_t n) {
  T* p = nullptr;
  cudaError_t e = cudaMalloc(&p, (n ? n : 1) * sizeof(T));
  if (e != cudaSuccess) throw CudaError(e, "cudaMalloc", __FILE__, __LINE__);
  return p;
}

}  // namespace

// Stencil (two face hops + Harmonic Balance partners), transpose positions
// and a greedy colouring in which no two cells of a colour share a row.
void build_exact_pattern(Handle& h) {
  const int N = h.m.N, F = h.m.F;
  std::vector<int> own(F), nei(F);
  if (F) {
    ICS_CUDA(cudaMemcpy(own.data(), h.m.own, F * sizeof(int), cudaMemcpyDeviceToHost));
    ICS_CUDA(cudaMemcpy(nei.data(), h.m.nei, F * sizeof(int), cudaMemcpyDeviceToHost));
  }
  // cyclic faces couple their cell with the partner cell (each pair of
  // faces gives both directions)
  std::vector<int> cyc(h.m.ncyc), bcell, bpart;
  if (h.m.ncyc) {
    const int B = h.m.B;
    bcell.resize(B);
    bpart.resize(B);
    ICS_CUDA(cudaMemcpy(cyc.data(), h.m.cyc_face, h.m.ncyc * sizeof(int), cudaMemcpyDeviceToHost));
    ICS_CUDA(cudaMemcpy(bcell.data(), h.m.bcell, B * sizeof(int), cudaMemcpyDeviceToHost));
    ICS_CUDA(cudaMemcpy(bpart.data(), h.m.bpartner, B * sizeof(int), cudaMemcpyDeviceToHost));
  }
  std::vector<int> aptr(N + 1, 0), adj(2 * (size_t)F + cyc.size());
  for (int f = 0; f < F; ++f) {
    aptr[own[f] + 1]++;
    aptr[nei[f] + 1]++;
  }
  for (int b : cyc) aptr[bcell[b] + 1]++;
  for (int c = 0; c < N; ++c) aptr[c + 1] += aptr[c];
  {
    std::vector<int> fill(aptr.begin(), aptr.end() - 1);
    for (int f = 0; f < F; ++f) {
      adj[fill[own[f]]++] = nei[f];
      adj[fill[nei[f]]++] = own[f];
    }
    for (int b : cyc) adj[fill[bcell[b]]++] = bpart[b];
  }
  const int nI = h.m.nInst, Nc = h.m.Nc;
  // cells with phase-lag cyclic faces -> their partners (CSR)
  std::vector<int> plagPtr, plagCells;
  if (h.m.plagMode && h.m.ncyc) {
    std::vector<int> pm(h.m.npatches), bpatch(h.m.B);
    ICS_CUDA(cudaMemcpy(pm.data(), h.m.plagMode, pm.size() * sizeof(int), cudaMemcpyDeviceToHost));
    ICS_CUDA(cudaMemcpy(bpatch.data(), h.m.bpatch, h.m.B * sizeof(int), cudaMemcpyDeviceToHost));
    plagPtr.assign(N + 1, 0);
    for (int b : cyc)
      if (pm[bpatch[b]]) plagPtr[bcell[b] + 1]++;
    for (int c = 0; c < N; ++c) plagPtr[c + 1] += plagPtr[c];
    plagCells.resize(plagPtr[N]);
    std::vector<int> fill(plagPtr.begin(), plagPtr.end() - 1);
    for (int b : cyc)
      if (pm[bpatch[b]]) plagCells[fill[bcell[b]]++] = bpart[b];
  }
  std::vector<int> ptr(N + 1, 0), col;
  col.reserve((size_t)N * 27);
  std::vector<int> mark(N, -1), row;
  for (int r = 0; r < N; ++r) {
    row.clear();
    auto add = [&](int c) {
      if (mark[c] != r) {
        mark[c] = r;
        row.push_back(c);
      }
    };
    add(r);
    for (int a = aptr[r]; a < aptr[r + 1]; ++a) {
      const int n1 = adj[a];
      add(n1);
      for (int b = aptr[n1]; b < aptr[n1 + 1]; ++b) add(adj[b]);
    }
    if (nI > 1) {
      const int cl = r % Nc;
      for (int K = 0; K < nI; ++K) add(K * Nc + cl);
      // phase-lag faces: the partner cells of every instance, and theirs
      // through the neighbours' gradients (rows within two hops)
      if (!plagCells.empty()) {
        auto addPl = [&](int c) {
          for (int e = plagPtr[c]; e < plagPtr[c + 1]; ++e) {
            const int cl2 = plagCells[e] % Nc;
            for (int K = 0; K < nI; ++K) add(K * Nc + cl2);
          }
        };
        addPl(r);
        for (int a = aptr[r]; a < aptr[r + 1]; ++a) addPl(adj[a]);
      }
    }
    std::sort(row.begin(), row.end());
    col.insert(col.end(), row.begin(), row.end());
    ptr[r + 1] = (int)col.size();
    // rows, columns and transpose positions are 32-bit; block entries are
    // addressed as (size_t) block * 25
    if (col.size() > (size_t)0x7fffffff) throw std::string("exact Jacobian stencil too large");
  }
  const size_t nnz = col.size();
  // transpose positions: entry (r, c) -> index of (c, r) in row c
  std::vector<int> tpos(nnz);
  for (int r = 0; r < N; ++r)
    for (int j = ptr[r]; j < ptr[r + 1]; ++j) {
      const int c = col[j];
      const int* b = col.data() + ptr[c];
      const int* e = col.data() + ptr[c + 1];
      const int* it = std::lower_bound(b, e, r);
      tpos[j] = (int)(it - col.data());
    }
  // greedy colouring: cells conflict when a row's stencil holds both, i.e.
  // the colours of every cell in the stencils of the rows of c's stencil
  // (the stencil relation is symmetric) are forbidden for c
  std::vector<int> colour(N, -1), seen;
  int ncol = 0;
  for (int c = 0; c < N; ++c) {
    for (int j = ptr[c]; j < ptr[c + 1]; ++j) {
      const int r = col[j];
      for (int q = ptr[r]; q < ptr[r + 1]; ++q) {
        const int t = colour[col[q]];
        if (t >= 0) {
          if ((int)seen.size() <= t) seen.resize(t + 1, -1);
          seen[t] = c;
        }
      }
    }
    int k = 0;
    while (k < (int)seen.size() && seen[k] == c) ++k;
    colour[c] = k;
    ncol = std::max(ncol, k + 1);
  }
  auto up = [&](const std::vector<int>& v) {
    int* p = xalloc<int>(v.size());
    if (!v.empty()) ICS_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice));
    return p;
  };
  h.xptr = up(ptr);
  h.xcol = up(col);
  h.xtpos = up(tpos);
  h.xcolour = up(colour);
  h.xnnz = (long long)nnz;
  h.xncol = ncol;
  h.xblk = xalloc<double>(nnz * 25);
}

void free_exact(Handle& h) {
  void* ptrs[] = {h.xptr, h.xcol, h.xtpos, h.xcolour, h.xblk};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  h.xptr = h.xcol = h.xtpos = h.xcolour = nullptr;
  h.xblk = nullptr;
  h.xnnz = 0;
  h.xncol = 0;
  h.haveExact = false;
}

void assemble_exact(Handle& h) {
  if (!h.xptr) build_exact_pattern(h);
  const int N = h.m.N;
  double* v = h.tv;
  double* jv = h.tv + 5ull * N;
  ICS_CUDA(cudaMemsetAsync(h.xblk, 0, (size_t)h.xnnz * 25 * sizeof(double), h.stream));
  for (int cid = 0; cid < h.xncol; ++cid)
    for (int k = 0; k < 5; ++k) {
      ICS_LAUNCH(h, ICS_K_EXACT, k_seed_colour<<<grid_for(N, 256), 256, 0, h.stream>>>(N, h.xcolour, cid, k, v));
      launch_residual_tangent(h, v, jv);
      ICS_LAUNCH(h, ICS_K_EXACT, k_exact_scatter<<<grid_for(N, 128), 128, 0, h.stream>>>(N, h.xptr, h.xcol, h.xcolour,
                                                                                          cid, k, jv, h.xblk));
    }
  ICS_CUDA(cudaGetLastError());
  h.haveExact = true;
}

void exact_vjp(Handle& h, const double* u, double* y) {
  ICS_LAUNCH(h, ICS_K_EXACT, k_exact_vjp<<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m.N, h.xptr, h.xcol, h.xtpos,
                                                                                      h.xblk, u, y));
  ICS_CUDA(cudaGetLastError());
}

void exact_jvp(Handle& h, const double* x, double* y) {
  ICS_LAUNCH(h, ICS_K_EXACT, k_exact_jvp<<<grid_for(h.m.N, 128), 128, 0, h.stream>>>(h.m.N, h.xptr, h.xcol, h.xblk,
                                                                                      x, y));
  ICS_CUDA(cudaGetLastError());
}

}  // namespace ics
