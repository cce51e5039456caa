// C ABI of the GB300 hot path and its host-side driver.
//
// ics_create uploads addressing and geometry once and builds, on the host:
//   - the cell->face CSR in face order (gathers accumulate in the order the
//     reference's face loops do),
//   - the sliced-ELL slot structure of the block Jacobian,
//   - the LU-SGS level schedule of the current cell numbering.
// Every later call works on device-resident state.  The host keeps only the
// scalar bookkeeping of the pseudo-time control (residualsIO history, SER,
// pseudotimeControl counters), mirroring setCoAndDeltaT.H and
// pseudotimeControl.C.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <cstring>
#include <new>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "blocks.cuh"
#include "ics_internal.cuh"

using namespace ics;

struct ics_handle_s {
  Handle h;
};

namespace ics {
double rho_l2(Handle& h);
double device_sum(Handle& h, const double* a, int n);

constexpr size_t EV_POOL = 8192;  // events; folded into the totals when full

// fold recorded event pairs into per-class totals (synchronises the stream)
static void prof_fold(Handle& h) {
  if (h.evUsed == 0) return;
  ICS_CUDA(cudaStreamSynchronize(h.stream));
  for (size_t p = 0; p < h.evKind.size(); ++p) {
    float t = 0;
    ICS_CUDA(cudaEventElapsedTime(&t, h.evPool[2 * p], h.evPool[2 * p + 1]));
    h.profMs[h.evKind[p]] += t;
    h.profN[h.evKind[p]] += 1;
  }
  h.evUsed = 0;
  h.evKind.clear();
}

Launch::Launch(Handle& hh, int k) : h(hh), kind(k) {
  h.launches++;
  if (!h.prof) return;
  if (h.evPool.empty()) {
    h.evPool.resize(EV_POOL);
    for (auto& e : h.evPool) ICS_CUDA(cudaEventCreate(&e));
  }
  if (h.evUsed + 2 > h.evPool.size()) prof_fold(h);
  ICS_CUDA(cudaEventRecord(h.evPool[h.evUsed], h.stream));
  stop = h.evPool[h.evUsed + 1];
  h.evKind.push_back(k);
  h.evUsed += 2;
}

Launch::~Launch() {
  if (stop) cudaEventRecord(stop, h.stream);
}
}  // namespace ics

namespace {

template <typename T>
T* dalloc(size_t n) {
  T* p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) throw CudaError(e, "cudaMalloc", __FILE__, __LINE__);
  ICS_CUDA(cudaMemset(p, 0, n * sizeof(T)));
  return p;
}

template <typename T>
T* upload(const std::vector<T>& v) {
  T* p = dalloc<T>(v.size());
  if (!v.empty()) ICS_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return p;
}

void dfree(void* p) {
  if (p) cudaFree(p);
}

void free_all(Handle& h) {
  DevMesh& m = h.m;
  void* ptrs[] = {m.own, m.nei, m.Sf, m.magSf, m.w, m.nodc, m.dOwn, m.dNei, m.dCC, m.nf, m.bnf, m.C, m.V,
                  m.bcell, m.bpatch, m.bSf, m.bmagSf, m.bdOwn, m.bdc, m.patches, m.cptr, m.cface, m.bptr,
                  m.bface, m.slot_base, m.scol, m.sface, m.nlow, m.nslot, m.fl_cells, m.rl_cells, m.fl_lptr,
                  m.rl_lptr, m.sweep_pad, m.sweep_ticket, h.W, h.W0, h.W00, h.Wprev, h.prim, h.pB, h.TB, h.UB, h.phiB, h.pseudoCo, h.rPDT,
                  h.ddtCoeff, h.q, h.bq, h.clin, h.grad, h.fflux, h.frec, h.flam, h.bjac, h.src, h.vcell,
                  h.fvisc, h.vsf2, h.vjac, m.dc, m.Dhb, m.mrfU, m.mrfOm, m.mrfBU, m.mrfBIn, m.plagMode, m.plagP, m.bpartner, m.bw, m.bdelta, m.bdNei,
                  m.bnodc, m.cyc_face, m.cyc_row, m.cyc_ptr, h.cblk, h.vjslotbuf, h.vjcellbuf, h.cfrec, h.tW, h.tprim, h.tq, h.tgrad, h.tflux, h.tvc, h.tfv, h.tv,
                  h.aF, h.aS, h.aQ, h.aG, h.aSrc, h.aVal, h.hbZoneBuf,
                  h.ss, h.ssB, h.srhoS, h.srhoS0, h.srhoS00, h.sgrad, h.sgradL, h.sface, h.sblk, h.sdg, h.srD,
                  h.ssrc, h.sFixed, h.sValue,
                  h.blk, h.dg,
                  h.dginv, h.rD, h.kv, h.kw, h.kx, h.kb, h.kt, h.dW, h.partials, h.counter, h.ks, h.scratch,
                  h.ibuf};
  drop_graphs(h);
  free_exact(h);
  free_cases(h);
  for (void* p : ptrs) dfree(p);
  for (cudaEvent_t e : h.evPool) cudaEventDestroy(e);
  if (h.tStart) cudaEventDestroy(h.tStart);
  if (h.tStop) cudaEventDestroy(h.tStop);
  if (h.ksHost) cudaFreeHost(h.ksHost);
  if (h.stream) cudaStreamDestroy(h.stream);
}

template <typename F>
int guard(ics_handle hh, F&& f) {
  if (!hh) return ICS_ERR_ARG;
  Handle& h = hh->h;
  try {
    return f(h);
  } catch (const CudaError& e) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s: %s (%s:%d)", e.what, cudaGetErrorString(e.e), e.file, e.line);
    h.err = buf;
    return e.e == cudaErrorMemoryAllocation ? ICS_ERR_NOMEM : ICS_ERR_CUDA;
  } catch (const std::string& s) {
    h.err = s;
    return ICS_ERR_ARG;
  } catch (const std::bad_alloc&) {
    h.err = "host allocation failed";
    return ICS_ERR_NOMEM;
  }
}

int validate_config(const ics_config* c, std::string& err) {
  if (c->flux_scheme < 0 || c->flux_scheme > 2) {
    err = "Unknown convectiveFluxScheme";
    return ICS_ERR_SCHEME;
  }
  if ((c->solver != ICS_SOLVER_GMRES && c->solver != ICS_SOLVER_SMOOTH) || c->preconditioner < 0 ||
      c->preconditioner > 2 || c->n_sweeps < 1) {
    err = "Unknown solver or preconditioner";
    return ICS_ERR_SCHEME;
  }
  if (c->viscous_lf_jacobian != 0 && c->viscous_lf_jacobian != 1) {
    err = "viscous_lf_jacobian must be 0 or 1";
    return ICS_ERR_ARG;
  }
  if (!(c->limiter_coeff > 0.0 && c->limiter_coeff <= 1.0)) {
    err = "cellLimited coefficient k must be in (0, 1]";
    return ICS_ERR_ARG;
  }
  const int rs[3] = {c->recon_rho, c->recon_U, c->recon_T};
  for (int r : rs)
    if (r < 0 || r > 4) {
      err = "Unknown reconstruction scheme";
      return ICS_ERR_SCHEME;
    }
  if (c->ddt_scheme < 0 || c->ddt_scheme > 2) {
    err = "Unknown ddt scheme";
    return ICS_ERR_SCHEME;
  }
  if (c->n_directions < 1 || c->n_directions > MAX_DIRS) {
    err = "nDirections out of range";
    return ICS_ERR_ARG;
  }
  if (c->precision != ICS_PREC_FP64 && c->precision != ICS_PREC_MIXED) {
    err = "unknown precision";
    return ICS_ERR_ARG;
  }
  if (!c->local_timestepping) {
    err = "global pseudo time stepping is not supported";
    return ICS_ERR_ARG;
  }
  if (!(c->R > 0) || !(c->Cp > c->R)) {
    err = "invalid thermo constants";
    return ICS_ERR_ARG;
  }
  return ICS_OK;
}

// Krylov and Jacobian storage sized for the current precision / nDirections
void ensure_workspace(Handle& h) {
  // Krylov vectors start on 256-byte boundaries (vectorised 16-byte access)
  const int p = prec(h);
  const int m = h.cfg.c.n_directions;
  const size_t eb = p == ICS_PREC_MIXED ? 4 : 8;
  const size_t n5 = 5ull * h.m.N;
  if (h.kvPrec != p || h.kvDirs < m) drop_graphs(h);  // captured pointers change
  if (h.kvPrec != p) {
    void* ptrs[] = {h.blk, h.dg, h.dginv, h.rD, h.kw, h.kx, h.kb, h.kt, h.kv};
    for (void* q : ptrs) dfree(q);
    // off-diagonal slots: factored in FP32, full in FP64 (blocks.cuh)
    h.blk = dalloc<char>((size_t)h.m.nslots * slot_words(p == ICS_PREC_MIXED) * 32 * eb);
    h.dg = dalloc<char>((size_t)h.m.nslices * 25 * 32 * eb);
    h.dginv = dalloc<char>((size_t)h.m.nslices * 25 * 32 * eb);
    h.rD = dalloc<char>((size_t)h.m.N * eb);
    h.kw = dalloc<char>(n5 * eb);
    h.kx = dalloc<char>(n5 * eb);
    h.kb = dalloc<char>(n5 * eb);
    h.kt = dalloc<char>(n5 * eb);
    h.kv = dalloc<char>(kstride(h) * eb * m);
    h.kvDirs = m;
    h.kvPrec = p;
    h.haveMatrix = false;
  } else if (h.kvDirs < m) {
    dfree(h.kv);
    h.kv = dalloc<char>(kstride(h) * eb * m);
    h.kvDirs = m;
  }
}

void build_mesh(Handle& h, const ics_mesh_desc* d) {
  DevMesh& m = h.m;
  const int N = d->n_cells, F = d->n_faces, B = d->n_bfaces;
  m.N = N;
  m.Nc = N;
  m.F = F;
  m.B = B;
  for (int k = 0; k < 3; ++k) m.solD[k] = d->solution_d[k];
  for (int f = 0; f < F; ++f) {
    const int o = d->owner[f], n = d->neighbour[f];
    if (o < 0 || n >= N || o >= n) throw std::string("faces must satisfy 0 <= owner < neighbour < n_cells");
    if (f > 0 && (o < d->owner[f - 1] || (o == d->owner[f - 1] && n <= d->neighbour[f - 1])))
      throw std::string("internal faces must be in upper-triangular order");
  }
  for (int b = 0; b < B; ++b)
    if (d->b_cell[b] < 0 || d->b_cell[b] >= N || d->b_patch[b] < 0 || d->b_patch[b] >= d->n_patches)
      throw std::string("boundary face addressing out of range");
  // geometry in SoA with the derived quantities the kernels use
  std::vector<double> Sf(3 * F), magSf(F), nf(3 * F), dOwn(3 * F), dNei(3 * F), dCC(3 * F);
  for (int f = 0; f < F; ++f) {
    const double s[3] = {d->Sf[3 * f], d->Sf[3 * f + 1], d->Sf[3 * f + 2]};
    const double ms = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    magSf[f] = ms;
    const int o = d->owner[f], n = d->neighbour[f];
    for (int k = 0; k < 3; ++k) {
      Sf[k * F + f] = s[k];
      nf[k * F + f] = s[k] / ms;
      dOwn[k * F + f] = d->Cf[3 * f + k] - d->C[3 * o + k];
      dNei[k * F + f] = d->Cf[3 * f + k] - d->C[3 * n + k];
      dCC[k * F + f] = d->C[3 * n + k] - d->C[3 * o + k];
    }
  }
  std::vector<double> bSf(3 * B), bmag(B), bnf(3 * B), bdOwn(3 * B);
  for (int b = 0; b < B; ++b) {
    const double s[3] = {d->b_Sf[3 * b], d->b_Sf[3 * b + 1], d->b_Sf[3 * b + 2]};
    const double ms = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    bmag[b] = ms;
    for (int k = 0; k < 3; ++k) {
      bSf[k * B + b] = s[k];
      bnf[k * B + b] = s[k] / ms;
      bdOwn[k * B + b] = d->b_Cf[3 * b + k] - d->C[3 * d->b_cell[b] + k];
    }
  }
  std::vector<double> C(3 * N);
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < 3; ++k) C[k * N + i] = d->C[3 * i + k];
  m.own = upload(std::vector<int>(d->owner, d->owner + F));
  m.nei = upload(std::vector<int>(d->neighbour, d->neighbour + F));
  m.Sf = upload(Sf);
  m.magSf = upload(magSf);
  m.nf = upload(nf);
  m.w = upload(std::vector<double>(d->weights, d->weights + F));
  m.nodc = upload(std::vector<double>(d->nonorth_delta_coeffs, d->nonorth_delta_coeffs + F));
  m.dc = upload(std::vector<double>(d->delta_coeffs, d->delta_coeffs + F));
  m.dOwn = upload(dOwn);
  m.dNei = upload(dNei);
  m.dCC = upload(dCC);
  m.C = upload(C);
  m.V = upload(std::vector<double>(d->V, d->V + N));
  m.bcell = upload(std::vector<int>(d->b_cell, d->b_cell + B));
  m.bpatch = upload(std::vector<int>(d->b_patch, d->b_patch + B));
  m.bSf = upload(bSf);
  m.bmagSf = upload(bmag);
  m.bnf = upload(bnf);
  m.bdOwn = upload(bdOwn);
  m.bdc = upload(std::vector<double>(d->b_delta_coeffs, d->b_delta_coeffs + B));
  std::vector<Patch> pts(std::max(1, d->n_patches));
  for (int p = 0; p < d->n_patches; ++p) {
    const ics_patch_desc& q = d->patches[p];
    pts[p].kind = q.kind;
    pts[p].is_wall = q.is_wall;
    pts[p].p = q.p;
    pts[p].T = q.T;
    for (int k = 0; k < 3; ++k) pts[p].U[k] = q.U[k];
    pts[p].p0 = q.p0;
    pts[p].T0 = q.T0;
    for (int k = 0; k < 9; ++k) pts[p].R[k] = q.rotation[k];
    if (q.kind < 0 || q.kind > ICS_PATCH_CYCLIC) throw std::string("unknown patch kind");
  }
  m.patches = upload(pts);
  m.npatches = d->n_patches;
  // coupled (cyclic) faces
  {
    std::vector<int> cycFaces;
    for (int b = 0; b < B; ++b)
      if (d->patches[d->b_patch[b]].kind == ICS_PATCH_CYCLIC) cycFaces.push_back(b);
    if (!cycFaces.empty()) {
      if (!d->b_partner || !d->b_weights || !d->b_nbr_d)
        throw std::string("cyclic patches need b_partner, b_weights and b_nbr_d");
      std::vector<int> partner(B, -1);
      std::vector<double> w(B, 1.0), delta(3 * (size_t)B, 0.0), nbrd(3 * (size_t)B, 0.0), nodc(B);
      for (int b = 0; b < B; ++b) nodc[b] = d->b_nonorth_delta_coeffs ? d->b_nonorth_delta_coeffs[b] : d->b_delta_coeffs[b];
      for (int b : cycFaces) {
        const int pc = d->b_partner[b];
        if (pc < 0 || pc >= N) throw std::string("cyclic face partner cell out of range");
        const double wb = d->b_weights[b];
        if (!(wb > 0.0 && wb < 1.0)) throw std::string("cyclic face weight outside (0, 1)");
        partner[b] = pc;
        w[b] = wb;
        for (int k = 0; k < 3; ++k) {
          const double nd = d->b_nbr_d[3 * b + k];
          nbrd[(size_t)k * B + b] = nd;
          delta[(size_t)k * B + b] = bdOwn[(size_t)k * B + b] - nd;
        }
      }
      // grouped by the owning cell for the row-owner coupling product
      std::stable_sort(cycFaces.begin(), cycFaces.end(),
                       [&](int a, int b2) { return d->b_cell[a] < d->b_cell[b2]; });
      std::vector<int> rows, ptr(1, 0);
      for (size_t i = 0; i < cycFaces.size(); ++i) {
        const int c = d->b_cell[cycFaces[i]];
        if (rows.empty() || rows.back() != c) {
          if (!rows.empty()) ptr.push_back((int)i);
          rows.push_back(c);
        }
      }
      ptr.push_back((int)cycFaces.size());
      m.bpartner = upload(partner);
      m.bw = upload(w);
      m.bdelta = upload(delta);
      m.bdNei = upload(nbrd);
      m.bnodc = upload(nodc);
      m.ncyc = (int)cycFaces.size();
      m.ncrow = (int)rows.size();
      m.cyc_face = upload(cycFaces);
      m.cyc_row = upload(rows);
      m.cyc_ptr = upload(ptr);
    }
  }
  // cell -> faces CSR in face order
  std::vector<int> cnt(N + 1, 0);
  for (int f = 0; f < F; ++f) {
    cnt[d->owner[f] + 1]++;
    cnt[d->neighbour[f] + 1]++;
  }
  for (int i = 0; i < N; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> cface(cnt[N]);
  {
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int f = 0; f < F; ++f) {
      cface[fill[d->owner[f]]++] = f;
      cface[fill[d->neighbour[f]]++] = ~f;
    }
  }
  m.cptr = upload(cnt);
  m.cface = upload(cface);
  std::vector<int> bcnt(N + 1, 0);
  for (int b = 0; b < B; ++b) bcnt[d->b_cell[b] + 1]++;
  for (int i = 0; i < N; ++i) bcnt[i + 1] += bcnt[i];
  std::vector<int> bface(B);
  {
    std::vector<int> fill(bcnt.begin(), bcnt.end() - 1);
    for (int b = 0; b < B; ++b) bface[fill[d->b_cell[b]]++] = b;
  }
  m.bptr = upload(bcnt);
  m.bface = upload(bface);
  // sliced-ELL: row c slots = its faces in face order (lower part first)
  const int ns = (N + SLICE - 1) / SLICE;
  m.nslices = ns;
  std::vector<int> slot_base(ns + 1, 0), nslot(N), nlow(N);
  for (int c = 0; c < N; ++c) {
    nslot[c] = cnt[c + 1] - cnt[c];
    int nl = 0;
    for (int e = cnt[c]; e < cnt[c + 1]; ++e) nl += cface[e] < 0;
    nlow[c] = nl;
  }
  for (int s = 0; s < ns; ++s) {
    int wmax = 0;
    for (int c = s * SLICE; c < std::min(N, (s + 1) * SLICE); ++c) wmax = std::max(wmax, nslot[c]);
    slot_base[s + 1] = slot_base[s] + wmax;
  }
  m.nslots = slot_base[ns];
  std::vector<int> scol((size_t)m.nslots * SLICE, -1), sface((size_t)m.nslots * SLICE, 0x7fffffff);
  for (int c = 0; c < N; ++c) {
    const int s = c / SLICE, lane = c % SLICE;
    // face order within a cell: neighbour-side faces (lower, col = owner
    // ascending) come before owner-side faces (upper, col = neighbour ascending)
    int t = 0;
    for (int e = cnt[c]; e < cnt[c + 1]; ++e) {
      const int code = cface[e];
      const int f = code >= 0 ? code : ~code;
      const int col = code >= 0 ? d->neighbour[f] : d->owner[f];
      const size_t idx = (size_t)(slot_base[s] + t) * SLICE + lane;
      scol[idx] = col;
      sface[idx] = code;
      ++t;
    }
  }
  // verify the slot column order (lower part ascending, then upper ascending)
  for (int c = 0; c < N; ++c) {
    const int s = c / SLICE, lane = c % SLICE;
    int prev = -1;
    for (int t = 0; t < nslot[c]; ++t) {
      const int col = scol[(size_t)(slot_base[s] + t) * SLICE + lane];
      if (col <= prev || (t < nlow[c]) != (col < c)) throw std::string("slot ordering invariant violated");
      prev = col;
    }
  }
  m.slot_base = upload(slot_base);
  m.scol = upload(scol);
  m.sface = upload(sface);
  m.nslot = upload(nslot);
  m.nlow = upload(nlow);
  // LU-SGS levels
  std::vector<int> lev(N, 0), rlev(N, 0);
  for (int c = 0; c < N; ++c)
    for (int e = cnt[c]; e < cnt[c + 1]; ++e)
      if (cface[e] < 0) lev[c] = std::max(lev[c], lev[d->owner[~cface[e]]] + 1);
  for (int c = N - 1; c >= 0; --c)
    for (int e = cnt[c]; e < cnt[c + 1]; ++e)
      if (cface[e] >= 0) rlev[c] = std::max(rlev[c], rlev[d->neighbour[cface[e]]] + 1);
  auto group = [&](const std::vector<int>& L, int& nl, std::vector<int>& ptr, std::vector<int>& cells,
                   std::vector<int>& cstart) {
    nl = 0;
    for (int v : L) nl = std::max(nl, v + 1);
    ptr.assign(nl + 1, 0);
    for (int v : L) ptr[v + 1]++;
    for (int l = 0; l < nl; ++l) ptr[l + 1] += ptr[l];
    cells.assign(N, 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int c = 0; c < N; ++c) cells[fill[L[c]]++] = c;
    cstart.assign(nl, -1);
    for (int l = 0; l < nl; ++l) {
      bool contig = true;
      for (int i = ptr[l] + 1; i < ptr[l + 1]; ++i)
        if (cells[i] != cells[i - 1] + 1) contig = false;
      if (contig && ptr[l + 1] > ptr[l]) cstart[l] = cells[ptr[l]];
    }
  };
  std::vector<int> fcells, rcells;
  group(lev, m.nfl, m.fl_ptr, fcells, m.fl_cstart);
  group(rlev, m.nrl, m.rl_ptr, rcells, m.rl_cstart);
  {
    const int a = m.fl_ptr[m.nfl - 1], b = m.fl_ptr[m.nfl];
    m.fuse_last = (b - a) == (m.rl_ptr[1] - m.rl_ptr[0]) &&
                  std::equal(fcells.begin() + a, fcells.begin() + b, rcells.begin() + m.rl_ptr[0]);
  }
  m.fl_cells = upload(fcells);
  m.rl_cells = upload(rcells);
  m.fl_lptr = upload(m.fl_ptr);
  // outputs of the sync-free sweeps (the schedules with many levels only)
  if (m.nfl > 2 && (long)N >= 2048L * m.nfl) m.sweep_pad = dalloc<double>(16ull * N);
  m.sweep_ticket = dalloc<unsigned int>(2);
  m.rl_lptr = upload(m.rl_ptr);
}

void alloc_state(Handle& h) {
  const int N = h.m.N, F = h.m.F, B = h.m.B;
  h.W = dalloc<double>(5ull * N);
  h.W0 = dalloc<double>(5ull * N);
  h.W00 = dalloc<double>(5ull * N);
  h.Wprev = dalloc<double>(5ull * N);
  h.prim = dalloc<double>(5ull * N);
  h.pB = dalloc<double>(B);
  h.TB = dalloc<double>(B);
  h.UB = dalloc<double>(3ull * B);
  h.phiB = dalloc<double>(B);
  h.pseudoCo = dalloc<double>(N);
  h.rPDT = dalloc<double>(N);
  h.ddtCoeff = dalloc<double>(N);
  h.q = dalloc<double>((size_t)NQ * N);
  h.bq = dalloc<double>((size_t)NQ * B);
  h.clin = dalloc<double>((size_t)N + B);
  h.grad = dalloc<double>((size_t)NQ * 3 * N);
  h.fflux = dalloc<double>(5ull * (F + B));
  h.frec = dalloc<double>(8ull * F);
  h.flam = dalloc<double>((size_t)F + B);
  if (h.m.ncyc) {
    h.cfrec = dalloc<double>(8ull * h.m.ncyc);
    h.cblk = dalloc<double>(25ull * h.m.ncyc);  // FP64 size; FP32 blocks use half
  }
  h.bjac = dalloc<double>(25ull * B);
  h.src = dalloc<double>(5ull * N);
  h.dW = dalloc<double>(5ull * N);
  h.partials = dalloc<double>((size_t)REDUCE_BLOCKS * 16);
  h.counter = dalloc<unsigned int>(MAX_INST + 4);
  h.ks = dalloc<KrylovScalars>(1);
  ICS_CUDA(cudaMallocHost(&h.ksHost, sizeof(KrylovScalars)));
  h.scratch = dalloc<double>(5ull * N + 8);
  h.ibuf = dalloc<int>((size_t)N + 8);
}

// sqrt(sum over instances of |s0|^2 + |s1|^2 + |v0|^2), scalars rho, rhoE and
// vector rhoU (setCoAndDeltaT.H:10-16; HB outerLoop.H:34-56)
double residual_norm(const std::vector<double>& r) {
  double s = 0;
  for (size_t J = 0; J < r.size() / 5; ++J) {
    const double* q = &r[5 * J];
    s += q[0] * q[0] + q[4] * q[4] + (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  }
  return std::sqrt(s);
}

// NVTX range around a phase of the pseudo iteration (visible in Nsight
// Systems timelines; a no-op without a tool attached)
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};

int do_residual(Handle& h, double* host_src) {
  Range rg("ics residual");
  // SER (setCoAndDeltaT.H:3-37) from the last two linear-solver initial residuals
  double ratio = 1.0;
  bool apply = false;
  if (h.cases.n) {
    // per case, as its own handle would (frozen cases: none)
    CaseSet& S = h.cases;
    for (int k = 0; k < S.n; ++k) {
      S.hser[k] = -1.0;
      if (S.frozen[k] || !S.initValid[k]) continue;
      const std::vector<double> in(&S.initRes[5 * k], &S.initRes[5 * k] + 5);
      if (S.ctl[k].corr != 1 && S.prevValid[k]) {
        const std::vector<double> pr(&S.prevRes[5 * k], &S.prevRes[5 * k] + 5);
        double r = residual_norm(pr) / residual_norm(in);
        S.hser[k] = std::max(std::min(r, h.cfg.c.pseudo_co_max_increase), h.cfg.c.pseudo_co_min_decrease);
      }
      std::copy(in.begin(), in.end(), &S.prevRes[5 * k]);
      S.prevValid[k] = 1;
    }
    case_upload_ser(h);
  } else if (h.initResValid) {
    const bool firstIter = h.ctl[0].corr == 1;
    if (!firstIter && h.prevResValid) {
      ratio = residual_norm(h.prevRes) / residual_norm(h.initRes);
      ratio = std::max(std::min(ratio, h.cfg.c.pseudo_co_max_increase), h.cfg.c.pseudo_co_min_decrease);
      apply = true;
    }
    h.prevRes = h.initRes;
    h.prevResValid = true;
  }
  launch_fields(h);
  launch_grad(h);
  launch_face_flux(h);
  if (h.cfg.c.viscous) {
    if (!h.vcell) {
      h.vcell = dalloc<double>(24ull * h.m.N);
      h.fvisc = dalloc<double>(8ull * (h.m.F + h.m.B));
      h.vsf2 = dalloc<double>((size_t)h.m.F + h.m.B);
      h.vjac = dalloc<double>(2ull * (h.m.F + h.m.B));
    }
    launch_viscous(h);
  }
  launch_residual(h, ratio, apply);
  h.haveFlux = true;
  h.lastRhoL2 = rho_l2(h);
  if (h.cases.n) case_l2(h);
  if (host_src) {
    ICS_CUDA(cudaMemcpyAsync(host_src, h.src, 5ull * h.m.N * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    for (size_t i = 0; i < 5ull * h.m.N; ++i)
      if (!std::isfinite(host_src[i])) {
        h.err = "non-finite residual";
        return ICS_ERR_NONFINITE;
      }
  }
  if (!std::isfinite(h.lastRhoL2)) {
    h.err = "non-finite residual";
    return ICS_ERR_NONFINITE;
  }
  return ICS_OK;
}

int do_jacobian(Handle& h) {
  Range rg("ics jacobian");
  if (!h.haveFlux) {
    h.err = "assemble_jacobian needs a residual evaluation first";
    return ICS_ERR_STATE;
  }
  ensure_workspace(h);
  ICS_CUDA(cudaMemsetAsync(&h.ks->status, 0, sizeof(int), h.stream));
  launch_jacobian(h);
  int st = 0;
  ICS_CUDA(cudaMemcpyAsync(&st, &h.ks->status, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
  ICS_CUDA(cudaStreamSynchronize(h.stream));
  h.haveMatrix = true;
  if (st) {
    h.err = "All diagonals of coupledMatrix are zero";
    return ICS_ERR_DIAG;
  }
  return ICS_OK;
}

int do_solve(Handle& h, ics_solver_perf* perf) {
  Range rg("ics gmres");
  if (!h.haveMatrix) {
    h.err = "solve_increment needs an assembled Jacobian";
    return ICS_ERR_STATE;
  }
  ensure_workspace(h);
  ICS_CUDA(cudaMemcpyAsync(h.Wprev, h.W, 5ull * h.m.N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
  ics_solver_perf p;
  if (h.cases.n) {
    CaseSet& S = h.cases;
    std::vector<int> cst;
    int st = gmres_cases(h, cst);
    std::memset(&p, 0, sizeof(p));
    for (int k = 0; k < 5; ++k) p.init_res[k] = p.final_res[k] = -VGREAT;
    bool conv = true;
    for (int k = 0; k < S.n; ++k) {
      if (S.frozen[k]) continue;
      S.initValid[k] = 1;
      std::memcpy(S.ctl[k].residuals, &S.initRes[5 * k], 5 * sizeof(double));
      for (int j = 0; j < 5; ++j) {
        p.init_res[j] = std::max(p.init_res[j], S.initRes[5 * k + j]);
        p.final_res[j] = std::max(p.final_res[j], S.finRes[5 * k + j]);
      }
      p.n_iterations = std::max(p.n_iterations, S.cycles[k]);
      if (cst[k] == ICS_ERR_NONFINITE && st == ICS_OK) st = ICS_ERR_NONFINITE;
      conv = conv && cst[k] == ICS_OK;
    }
    p.converged = conv && st == ICS_OK;
    h.haveIncrement = true;
    if (perf) *perf = p;
    if (st) h.err = st == ICS_ERR_TIMEOUT ? "LU-SGS sweep wait gave up" : "non-finite Krylov residual in a case";
    return st;
  }
  const int st = gmres_solve(h, &p, h.initRes);
  h.haveIncrement = true;
  h.initResValid = true;
  for (int J = 0; J < h.m.nInst; ++J) std::memcpy(h.ctl[J].residuals, &h.initRes[5 * J], 5 * sizeof(double));
  if (perf) *perf = p;
  if (st) h.err = st == ICS_ERR_BREAKDOWN ? "zero Krylov norm" : "non-finite Krylov residual";
  return st;
}

int do_update(Handle& h, ics_iter_stats* s) {
  Range rg("ics update");
  if (!h.haveIncrement) {
    h.err = "update_fields needs a solved increment";
    return ICS_ERR_STATE;
  }
  launch_bound_local_timestep(h);
  h.haveExact = false;
  int* bounded = h.ibuf + h.m.N;
  ICS_CUDA(cudaMemsetAsync(bounded, 0, sizeof(int), h.stream));
  launch_update(h, bounded);
  launch_bc(h);
  int nb = 0;
  ICS_CUDA(cudaMemcpyAsync(&nb, bounded, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
  ICS_CUDA(cudaStreamSynchronize(h.stream));
  h.haveIncrement = false;
  if (s) {
    s->bounded_cells = nb;
    s->rho_l2_residual = h.lastRhoL2;
  }
  return ICS_OK;
}

// pseudotimeControl::criteriaSatisfied (pseudotimeControl.C), the residuals
// being the initial residuals of the last linear solve
bool criteria_satisfied(const Handle& h, Handle::Control& q) {
  const ics_config& c = h.cfg.c;
  const bool finalIter = q.converged || (q.corr == c.n_pseudo_corr);
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
  const bool absCheck = mx < c.pseudo_tol;
  const bool relCheck = !storeIni && mrel < c.pseudo_tol_rel;
  return (q.corr >= c.n_pseudo_corr_min) && (absCheck || relCheck);
}

// pseudotimeControl::loop (pseudotimeControl.C:159-241) for one control
bool pseudo_loop_one(const Handle& h, Handle::Control& q) {
  const bool steady = h.cfg.c.ddt_scheme == ICS_DDT_STEADY;
  q.corr++;
  if (!steady && q.corr == h.cfg.c.n_pseudo_corr + 1) {
    q.corr = 0;
    return false;
  }
  bool completed = false;
  if (q.converged || criteria_satisfied(h, q)) {
    if (q.converged) {
      q.corr = 0;
      q.converged = false;
      completed = true;
    } else {
      q.converged = true;
    }
  }
  return !completed;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

void ics_default_config(ics_config* c) {
  if (!c) return;
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

int ics_create(const ics_mesh_desc* mesh, const ics_config* cfg, ics_handle* out) {
  if (!mesh || !cfg || !out || mesh->n_cells <= 0 || mesh->n_faces < 0 || mesh->n_bfaces < 0 ||
      mesh->n_patches < 0 || (mesh->n_faces && (!mesh->owner || !mesh->neighbour || !mesh->Sf || !mesh->Cf)) ||
      !mesh->C || !mesh->V)
    return ICS_ERR_ARG;
  *out = nullptr;
  ics_handle hh = new (std::nothrow) ics_handle_s();
  if (!hh) return ICS_ERR_NOMEM;
  std::string err;
  int st = validate_config(cfg, err);
  if (st) {
    delete hh;
    return st;
  }
  Handle& h = hh->h;
  h.cfg.c = *cfg;
  h.cfg.Cv = cfg->Cp - cfg->R;
  h.cfg.gamma = cfg->Cp / h.cfg.Cv;
  h.m.gamma = h.cfg.gamma;
  h.m.limWiden = 1.0 / cfg->limiter_coeff - 1.0;
  st = guard(hh, [&](Handle& hd) {
    ICS_CUDA(cudaGetDevice(&hd.device));
    ICS_CUDA(cudaStreamCreateWithFlags(&hd.stream, cudaStreamNonBlocking));
    build_mesh(hd, mesh);
    alloc_state(hd);
    ensure_workspace(hd);
    std::vector<double> co(hd.m.N, cfg->pseudo_co_num);
    ICS_CUDA(cudaMemcpy(hd.pseudoCo, co.data(), co.size() * sizeof(double), cudaMemcpyHostToDevice));
    return ICS_OK;
  });
  if (st) {
    free_all(h);
    delete hh;
    return st;
  }
  *out = hh;
  return ICS_OK;
}

int ics_destroy(ics_handle hh) {
  if (!hh) return ICS_ERR_ARG;
  free_all(hh->h);
  delete hh;
  return ICS_OK;
}

int ics_set_config(ics_handle hh, const ics_config* cfg) {
  if (!hh || !cfg) return ICS_ERR_ARG;
  std::string err;
  const int st = validate_config(cfg, err);
  if (st) {
    hh->h.err = err;
    return st;
  }
  if (hh->h.m.nInst > 1 && (cfg->ddt_scheme != ICS_DDT_STEADY || cfg->solver != ICS_SOLVER_GMRES)) {
    hh->h.err = "Harmonic Balance needs steadyState ddt and the GMRES solver";
    return ICS_ERR_ARG;
  }
  if (hh->h.cases.n && cfg->solver != ICS_SOLVER_GMRES) {
    hh->h.err = "stacked cases need the GMRES solver";
    return ICS_ERR_ARG;
  }

  return guard(hh, [&](Handle& h) {
    const bool structural = cfg->precision != h.cfg.c.precision || cfg->n_directions != h.cfg.c.n_directions;
    // the Jacobian storage depends on the precision (factored FP32 / full FP64 slots),
    // and the factored FP32 slots apply gamma when they are used, so a new gamma
    // would meet diagonal blocks assembled under the old one
    const bool precChange = cfg->precision != h.cfg.c.precision;
    const bool gammaChange = cfg->Cp != h.cfg.c.Cp || cfg->R != h.cfg.c.R;
    h.cfg.c = *cfg;
    h.cfg.Cv = cfg->Cp - cfg->R;
    h.cfg.gamma = cfg->Cp / h.cfg.Cv;
    h.m.gamma = h.cfg.gamma;
    h.m.limWiden = 1.0 / cfg->limiter_coeff - 1.0;
    h.haveExact = false;
    if (structural) ensure_workspace(h);
    if (precChange || gammaChange) h.haveMatrix = false;  // reassembled by the next iteration
    return ICS_OK;
  });
}

int ics_last_error(ics_handle hh, char* buf, int32_t len) {
  if (!hh || !buf || len <= 0) return ICS_ERR_ARG;
  std::snprintf(buf, len, "%s", hh->h.err.c_str());
  return ICS_OK;
}

int ics_set_primitive(ics_handle hh, const double* p, const double* U, const double* T) {
  if (!p || !U || !T) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    const size_t N = h.m.N;
    ICS_CUDA(cudaMemcpyAsync(h.scratch, p, N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    ICS_CUDA(cudaMemcpyAsync(h.scratch + N, U, 3 * N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    ICS_CUDA(cudaMemcpyAsync(h.scratch + 4 * N, T, N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    launch_set_primitive(h);
    ICS_CUDA(cudaMemcpyAsync(h.W0, h.W, 5 * N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
    ICS_CUDA(cudaMemcpyAsync(h.W00, h.W, 5 * N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    h.timeIndex = 0;
    h.haveFlux = h.haveMatrix = h.haveIncrement = h.haveExact = false;
    return ICS_OK;
  });
}

int ics_set_boundary_state(ics_handle hh, const double* pb, const double* Ub, const double* Tb, const double* phib) {
  return guard(hh, [&](Handle& h) {
    const size_t B = h.m.B;
    h.haveExact = false;
    if (pb) ICS_CUDA(cudaMemcpy(h.pB, pb, B * sizeof(double), cudaMemcpyHostToDevice));
    if (Tb) ICS_CUDA(cudaMemcpy(h.TB, Tb, B * sizeof(double), cudaMemcpyHostToDevice));
    if (phib) ICS_CUDA(cudaMemcpy(h.phiB, phib, B * sizeof(double), cudaMemcpyHostToDevice));
    if (Ub) {
      std::vector<double> t(3 * B);
      for (size_t b = 0; b < B; ++b)
        for (int k = 0; k < 3; ++k) t[k * B + b] = Ub[3 * b + k];
      ICS_CUDA(cudaMemcpy(h.UB, t.data(), 3 * B * sizeof(double), cudaMemcpyHostToDevice));
    }
    return ICS_OK;
  });
}

int ics_get_boundary_state(ics_handle hh, double* pb, double* Ub, double* Tb, double* phib) {
  return guard(hh, [&](Handle& h) {
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    const size_t B = h.m.B;
    if (pb) ICS_CUDA(cudaMemcpy(pb, h.pB, B * sizeof(double), cudaMemcpyDeviceToHost));
    if (Tb) ICS_CUDA(cudaMemcpy(Tb, h.TB, B * sizeof(double), cudaMemcpyDeviceToHost));
    if (phib) ICS_CUDA(cudaMemcpy(phib, h.phiB, B * sizeof(double), cudaMemcpyDeviceToHost));
    if (Ub) {
      std::vector<double> t(3 * B);
      ICS_CUDA(cudaMemcpy(t.data(), h.UB, 3 * B * sizeof(double), cudaMemcpyDeviceToHost));
      for (size_t b = 0; b < B; ++b)
        for (int k = 0; k < 3; ++k) Ub[3 * b + k] = t[k * B + b];
    }
    return ICS_OK;
  });
}

int ics_get_state(ics_handle hh, double* W, double* p, double* U, double* T) {
  return guard(hh, [&](Handle& h) {
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    const size_t N = h.m.N;
    if (W) ICS_CUDA(cudaMemcpy(W, h.W, 5 * N * sizeof(double), cudaMemcpyDeviceToHost));
    if (p || U || T) {
      std::vector<double> pr(5 * N);
      ICS_CUDA(cudaMemcpy(pr.data(), h.prim, 5 * N * sizeof(double), cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < N; ++i) {
        if (p) p[i] = pr[i];
        if (T) T[i] = pr[N + i];
        if (U)
          for (int k = 0; k < 3; ++k) U[3 * i + k] = pr[(2 + k) * N + i];
      }
    }
    return ICS_OK;
  });
}

int ics_set_conservative(ics_handle hh, const double* W, int32_t set_old) {
  if (!W) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    const size_t N = h.m.N;
    ICS_CUDA(cudaMemcpyAsync(h.W, W, 5 * N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    launch_derive_primitive(h);
    h.haveExact = false;
    if (set_old) {
      ICS_CUDA(cudaMemcpyAsync(h.W0, h.W, 5 * N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
      ICS_CUDA(cudaMemcpyAsync(h.W00, h.W, 5 * N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
    }
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    return ICS_OK;
  });
}

int ics_set_pseudo_co(ics_handle hh, const double* co) {
  if (!co) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    ICS_CUDA(cudaMemcpy(h.pseudoCo, co, h.m.N * sizeof(double), cudaMemcpyHostToDevice));
    return ICS_OK;
  });
}

int ics_get_pseudo_co(ics_handle hh, double* co, double* rdt) {
  return guard(hh, [&](Handle& h) {
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (co) ICS_CUDA(cudaMemcpy(co, h.pseudoCo, h.m.N * sizeof(double), cudaMemcpyDeviceToHost));
    if (rdt) ICS_CUDA(cudaMemcpy(rdt, h.rPDT, h.m.N * sizeof(double), cudaMemcpyDeviceToHost));
    return ICS_OK;
  });
}

int ics_calc_flux(ics_handle hh, double* phi, double* phiU, double* phiE) {
  return guard(hh, [&](Handle& h) {
    launch_fields(h);
    launch_grad(h);
    launch_face_flux(h);
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    const size_t FB = (size_t)h.m.F + h.m.B;
    std::vector<double> t(5 * FB);
    ICS_CUDA(cudaMemcpy(t.data(), h.fflux, 5 * FB * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t f = 0; f < FB; ++f) {
      if (phi) phi[f] = t[f];
      if (phiU)
        for (int k = 0; k < 3; ++k) phiU[3 * f + k] = t[(1 + k) * FB + f];
      if (phiE) phiE[f] = t[4 * FB + f];
    }
    return ICS_OK;
  });
}

int ics_residual(ics_handle hh, double* source) {
  return guard(hh, [&](Handle& h) { return do_residual(h, source); });
}

int ics_assemble_jacobian(ics_handle hh) {
  return guard(hh, [&](Handle& h) { return do_jacobian(h); });
}

int ics_get_jacobian(ics_handle hh, double* diag, double* lower, double* upper) {
  return guard(hh, [&](Handle& h) {
    if (!h.haveMatrix) {
      h.err = "no assembled Jacobian";
      return ICS_ERR_STATE;
    }
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    const DevMesh& m = h.m;
    const bool mixed = h.jacPrecision == ICS_PREC_MIXED;
    const size_t eb = mixed ? 4 : 8;
    // the off-diagonal slots are stored factored: expand them on the device
    std::vector<double> blk((size_t)m.nslots * 25 * 32);
    std::vector<char> dg((size_t)m.nslices * 25 * 32 * eb);
    double* tmp = nullptr;
    ICS_CUDA(cudaMalloc(&tmp, blk.size() * sizeof(double)));
    launch_expand_slots(h, tmp);
    cudaError_t e1 = cudaMemcpyAsync(blk.data(), tmp, blk.size() * sizeof(double), cudaMemcpyDeviceToHost, h.stream);
    if (e1 == cudaSuccess) e1 = cudaStreamSynchronize(h.stream);  // the handle's stream does not block
    cudaFree(tmp);
    ICS_CUDA(e1);
    ICS_CUDA(cudaMemcpy(dg.data(), h.dg, dg.size(), cudaMemcpyDeviceToHost));
    std::vector<int> sb(m.nslices + 1), sface((size_t)m.nslots * 32), nsl(m.N);
    ICS_CUDA(cudaMemcpy(sb.data(), m.slot_base, sb.size() * sizeof(int), cudaMemcpyDeviceToHost));
    ICS_CUDA(cudaMemcpy(sface.data(), m.sface, sface.size() * sizeof(int), cudaMemcpyDeviceToHost));
    ICS_CUDA(cudaMemcpy(nsl.data(), m.nslot, nsl.size() * sizeof(int), cudaMemcpyDeviceToHost));
    auto get = [&](const std::vector<char>& a, size_t idx) {
      return mixed ? (double)((const float*)a.data())[idx] : ((const double*)a.data())[idx];
    };
    for (int c = 0; c < m.N; ++c) {
      const int s = c / 32, lane = c % 32;
      if (diag)
        for (int k = 0; k < 25; ++k) diag[25 * c + k] = get(dg, ((size_t)s * 25 + k) * 32 + lane);
      for (int t = 0; t < nsl[c]; ++t) {
        const int code = sface[(size_t)(sb[s] + t) * 32 + lane];
        const int f = code >= 0 ? code : ~code;
        double* dst = code >= 0 ? upper : lower;  // owner row holds upper_f
        if (!dst) continue;
        for (int k = 0; k < 25; ++k) dst[25 * f + k] = blk[((size_t)(sb[s] + t) * 25 + k) * 32 + lane];
      }
    }
    return ICS_OK;
  });
}

int ics_matrix_mul(ics_handle hh, const double* x, double* y) {
  if (!x || !y) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    if (!h.haveMatrix) {
      h.err = "no assembled Jacobian";
      return ICS_ERR_STATE;
    }
    const size_t n5 = 5ull * h.m.N;
    ICS_CUDA(cudaMemcpyAsync(h.scratch, x, n5 * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    to_vec(h, h.scratch, h.kw);
    spmv(h, h.kw, h.kt);
    from_vec(h, h.kt, h.scratch);
    ICS_CUDA(cudaMemcpyAsync(y, h.scratch, n5 * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    return ICS_OK;
  });
}

int ics_precondition(ics_handle hh, double* r) {
  if (!r) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    if (!h.haveMatrix) {
      h.err = "no assembled Jacobian";
      return ICS_ERR_STATE;
    }
    const size_t n5 = 5ull * h.m.N;
    ICS_CUDA(cudaMemsetAsync(&h.ks->status, 0, sizeof(int), h.stream));
    ICS_CUDA(cudaMemcpyAsync(h.scratch, r, n5 * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    to_vec(h, h.scratch, h.kw);
    precondition(h, h.kw);
    from_vec(h, h.kw, h.scratch);
    ICS_CUDA(cudaMemcpyAsync(r, h.scratch, n5 * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
    int st = 0;
    ICS_CUDA(cudaMemcpyAsync(&st, &h.ks->status, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (st & 8) {
      h.err = "a sync-free LU-SGS sweep gave up waiting";
      return ICS_ERR_TIMEOUT;
    }
    return ICS_OK;
  });
}

int ics_solve_increment(ics_handle hh, ics_solver_perf* perf, double* dW) {
  return guard(hh, [&](Handle& h) {
    const int st = do_solve(h, perf);
    if (dW) {
      ICS_CUDA(cudaMemcpyAsync(dW, h.dW, 5ull * h.m.N * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
      ICS_CUDA(cudaStreamSynchronize(h.stream));
    }
    return st;
  });
}

int ics_update_fields(ics_handle hh, ics_iter_stats* stats) {
  return guard(hh, [&](Handle& h) { return do_update(h, stats); });
}

int ics_pseudo_iteration(ics_handle hh, ics_iter_stats* stats) {
  return guard(hh, [&](Handle& h) {
    Range rg("ics pseudo iteration");
    ics_iter_stats s;
    std::memset(&s, 0, sizeof(s));
    int r = do_residual(h, nullptr);
    if (r) return r;
    r = do_jacobian(h);
    if (r) return r;
    const int sv = do_solve(h, &s.perf);
    if (sv && sv != ICS_ERR_BREAKDOWN) return sv;
    const int u = do_update(h, &s);
    s.pseudo_co_mean = device_sum(h, h.pseudoCo, h.m.N) / h.m.N;
    s.rho_l2_residual = h.lastRhoL2;
    s.status = sv ? sv : u;
    if (stats) *stats = s;
    return u;
  });
}

int ics_set_cases(ics_handle hh, int32_t n_cases, const int32_t* case_start) {
  return guard(hh, [&](Handle& h) {
    set_cases(h, n_cases, case_start);
    return ICS_OK;
  });
}

int ics_case_stats(ics_handle hh, double* rho_l2_out, int32_t* gmres_cycles, int32_t* frozen) {
  return guard(hh, [&](Handle& h) {
    const CaseSet& S = h.cases;
    if (!S.n) {
      h.err = "the handle holds no stacked cases";
      return ICS_ERR_STATE;
    }
    for (int k = 0; k < S.n; ++k) {
      if (rho_l2_out) rho_l2_out[k] = std::sqrt(S.hl2[k]);
      if (gmres_cycles) gmres_cycles[k] = S.cycles[k];
      if (frozen) frozen[k] = S.frozen[k];
    }
    return ICS_OK;
  });
}

int ics_pseudo_iteration_batch(ics_handle* hs, int32_t n, ics_iter_stats* stats, int32_t* status) {
  if (!hs || n < 0) return ICS_ERR_ARG;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (!hs[i] || hs[i] == hs[j]) return ICS_ERR_ARG;  // one thread per handle: no repeats
  std::atomic<int> next(0);
  std::vector<int> st(n, ICS_OK);
  auto work = [&]() {
    for (int i = next++; i < n; i = next++) st[i] = ics_pseudo_iteration(hs[i], stats ? &stats[i] : nullptr);
  };
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min<unsigned>(nt ? nt : 4, (unsigned)n));
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < nt; ++t) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  int first = ICS_OK;
  for (int i = 0; i < n; ++i) {
    if (status) status[i] = st[i];
    if (first == ICS_OK && st[i] != ICS_OK) first = st[i];
  }
  return first;
}

int ics_begin_time_step(ics_handle hh) {
  return guard(hh, [&](Handle& h) {
    const size_t n5 = 5ull * h.m.N;
    const bool steady = h.cfg.c.ddt_scheme == ICS_DDT_STEADY;
    if (h.timeIndex == 0) {
      ICS_CUDA(cudaMemcpyAsync(h.W0, h.W, n5 * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
      ICS_CUDA(cudaMemcpyAsync(h.W00, h.W, n5 * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
    } else {
      ICS_CUDA(cudaMemcpyAsync(h.W00, h.W0, n5 * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
      ICS_CUDA(cudaMemcpyAsync(h.W0, h.W, n5 * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
    }
    if (h.scalarOn) {
      const size_t N = h.m.N;
      ICS_CUDA(cudaMemcpyAsync(h.srhoS00, h.timeIndex == 0 ? h.srhoS : h.srhoS0, N * sizeof(double),
                               cudaMemcpyDeviceToDevice, h.stream));
      ICS_CUDA(cudaMemcpyAsync(h.srhoS0, h.srhoS, N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
    }
    // dbnsFoam outerLoop.H:6: the frame velocity on the zones' boundary faces
    launch_mrf_bc(h);
    h.timeIndex++;
    h.haveExact = false;
    if (!steady) {
      h.initResValid = false;
      h.prevResValid = false;
      std::fill(h.cases.initValid.begin(), h.cases.initValid.end(), 0);
      std::fill(h.cases.prevValid.begin(), h.cases.prevValid.end(), 0);
    }
    std::fill(h.cases.frozen.begin(), h.cases.frozen.end(), 0);
    if (h.cfg.c.reset_pseudo) {
      std::vector<double> co(h.m.N, h.cfg.c.pseudo_co_num);
      ICS_CUDA(cudaMemcpyAsync(h.pseudoCo, co.data(), co.size() * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    }
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    return ICS_OK;
  });
}

int ics_profile(ics_handle hh, int32_t enable) {
  return guard(hh, [&](Handle& h) {
    if (enable) {
      ICS_CUDA(cudaStreamSynchronize(h.stream));
      h.evUsed = 0;
      h.evKind.clear();
      for (int k = 0; k < ICS_K_COUNT; ++k) {
        h.profMs[k] = 0;
        h.profN[k] = 0;
      }
      h.prof = true;
    } else {
      h.prof = false;
      prof_fold(h);
    }
    return ICS_OK;
  });
}

int ics_profile_read(ics_handle hh, int32_t kind, double* ms, int64_t* launches) {
  if (kind < 0 || kind >= ICS_K_COUNT) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    prof_fold(h);
    if (ms) *ms = h.profMs[kind];
    if (launches) *launches = h.profN[kind];
    return ICS_OK;
  });
}

int ics_launch_count(ics_handle hh, int64_t* launches) {
  if (!launches) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    *launches = h.launches;
    return ICS_OK;
  });
}

int ics_timer_start(ics_handle hh) {
  return guard(hh, [&](Handle& h) {
    if (!h.tStart) {
      ICS_CUDA(cudaEventCreate(&h.tStart));
      ICS_CUDA(cudaEventCreate(&h.tStop));
    }
    ICS_CUDA(cudaEventRecord(h.tStart, h.stream));
    return ICS_OK;
  });
}

int ics_timer_stop(ics_handle hh, double* ms) {
  if (!ms) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    if (!h.tStart) return ICS_ERR_STATE;
    ICS_CUDA(cudaEventRecord(h.tStop, h.stream));
    ICS_CUDA(cudaEventSynchronize(h.tStop));
    float t = 0;
    ICS_CUDA(cudaEventElapsedTime(&t, h.tStart, h.tStop));
    *ms = t;
    return ICS_OK;
  });
}

// failure-detection probe ------------------------------------------------------
int ics_test_sweep_timeout(ics_handle hh, int32_t skip_row, int32_t spin_limit) {
  if (!hh || spin_limit < 1) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    const int N = h.m.N;
    if (!h.haveMatrix) {
      h.err = "test_sweep_timeout needs an assembled Jacobian";
      return ICS_ERR_STATE;
    }
    if (skip_row < 0 || skip_row >= N) return ICS_ERR_ARG;
    if (!h.m.sweep_pad) h.m.sweep_pad = dalloc<double>(16ull * N);  // schedules with few levels
    // the forward level order without skip_row
    std::vector<int> order(N);
    ICS_CUDA(cudaMemcpy(order.data(), h.m.fl_cells, N * sizeof(int), cudaMemcpyDeviceToHost));
    order.erase(std::remove(order.begin(), order.end(), (int)skip_row), order.end());
    if ((int)order.size() != N - 1) return ICS_ERR_ARG;
    ICS_CUDA(cudaMemcpy(h.ibuf, order.data(), (N - 1) * sizeof(int), cudaMemcpyHostToDevice));
    ICS_CUDA(cudaMemsetAsync(&h.ks->status, 0, sizeof(int), h.stream));
    sweep_probe(h, h.ibuf, N - 1, spin_limit);
    int st = 0;
    ICS_CUDA(cudaMemcpyAsync(&st, &h.ks->status, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (st & 8) {
      h.err = "a sync-free sweep wait gave up (as the probe intends)";
      return ICS_ERR_TIMEOUT;
    }
    return ICS_OK;
  });
}

// checkpoint / resume ----------------------------------------------------------
// Raw binary: a fixed header, then the arrays in a fixed order.  Everything
// the next pseudo iteration reads is included (state, old time levels,
// primitives, boundary values, pseudo Courant numbers, SER and pseudotime
// control state, the passive scalar), so a resumed run continues bit for bit.
namespace {
struct CkptHeader {
  char magic[8];
  int32_t version, N, F, B, nInst, scalarOn, timeIndex, initResValid, prevResValid, nres;
  double lastRhoL2;
};
constexpr int32_t CKPT_VERSION = 2;

struct CkptIO {
  Handle& h;
  char* out;
  const char* in;
  size_t pos = 0;
  void bytes(void* host, size_t n) {
    if (out) std::memcpy(out + pos, host, n);
    if (in) std::memcpy(host, in + pos, n);
    pos += n;
  }
  void dev(double* d, size_t n) {
    const size_t nb = n * sizeof(double);
    if (out) ICS_CUDA(cudaMemcpy(out + pos, d, nb, cudaMemcpyDeviceToHost));
    if (in) ICS_CUDA(cudaMemcpy(d, in + pos, nb, cudaMemcpyHostToDevice));
    pos += nb;
  }
};

size_t ckpt_walk(Handle& h, CkptHeader& hd, char* out, const char* in) {
  CkptIO io{h, out, in};
  io.bytes(&hd, sizeof(hd));
  const size_t N = h.m.N, B = h.m.B;
  io.dev(h.W, 5 * N);
  io.dev(h.W0, 5 * N);
  io.dev(h.W00, 5 * N);
  io.dev(h.prim, 5 * N);
  io.dev(h.pB, B);
  io.dev(h.TB, B);
  io.dev(h.UB, 3 * B);
  io.dev(h.phiB, B);
  io.dev(h.pseudoCo, N);
  io.dev(h.rPDT, N);  // the dual-time residual term rounds with the previous 1/dtau
  const size_t nres = 5 * (size_t)h.m.nInst;
  if (in) {
    h.initRes.resize(nres);
    h.prevRes.resize(nres);
  }
  std::vector<double> pad(nres, 0.0);
  io.bytes(h.initRes.size() == nres ? h.initRes.data() : pad.data(), nres * sizeof(double));
  io.bytes(h.prevRes.size() == nres ? h.prevRes.data() : pad.data(), nres * sizeof(double));
  for (auto& q : h.ctl) {
    int32_t v[3] = {q.corr, q.converged ? 1 : 0, q.firstIteration ? 1 : 0};
    io.bytes(v, sizeof(v));
    if (in) {
      q.corr = v[0];
      q.converged = v[1] != 0;
      q.firstIteration = v[2] != 0;
    }
    io.bytes(q.residuals, sizeof(q.residuals));
    io.bytes(q.initResiduals, sizeof(q.initResiduals));
  }
  if (h.scalarOn) {
    io.dev(h.ss, N);
    io.dev(h.ssB, B);
    io.dev(h.srhoS, N);
    io.dev(h.srhoS0, N);
    io.dev(h.srhoS00, N);
  }
  return io.pos;
}

CkptHeader ckpt_header(const Handle& h) {
  CkptHeader hd;
  std::memset(&hd, 0, sizeof(hd));
  std::memcpy(hd.magic, "ICSCKPT", 7);
  hd.version = CKPT_VERSION;
  hd.N = h.m.N;
  hd.F = h.m.F;
  hd.B = h.m.B;
  hd.nInst = h.m.nInst;
  hd.scalarOn = h.scalarOn ? 1 : 0;
  hd.timeIndex = h.timeIndex;
  hd.initResValid = h.initResValid ? 1 : 0;
  hd.prevResValid = h.prevResValid ? 1 : 0;
  hd.nres = 5 * h.m.nInst;
  hd.lastRhoL2 = h.lastRhoL2;
  return hd;
}
}  // namespace

int ics_checkpoint_size(ics_handle hh, int64_t* bytes) {
  if (!hh || !bytes) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    CkptHeader hd = ckpt_header(h);
    // a dry walk counts the bytes
    size_t n = sizeof(hd);
    const size_t N = h.m.N, B = h.m.B;
    n += sizeof(double) * (20 * N + 6 * B + 2 * N);
    n += 2 * sizeof(double) * 5 * h.m.nInst;
    n += h.ctl.size() * (3 * sizeof(int32_t) + 10 * sizeof(double));
    if (h.scalarOn) n += sizeof(double) * (4 * N + B);
    *bytes = (int64_t)n;
    return ICS_OK;
  });
}

int ics_save_checkpoint(ics_handle hh, void* buf, int64_t bytes) {
  if (!hh || !buf) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    if (h.cases.n) {
      h.err = "checkpoints do not carry the per-case controls of stacked cases";
      return ICS_ERR_ARG;
    }
    int64_t need = 0;
    ics_checkpoint_size(hh, &need);
    if (bytes < need) {
      h.err = "checkpoint buffer too small";
      return ICS_ERR_ARG;
    }
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    CkptHeader hd = ckpt_header(h);
    ckpt_walk(h, hd, (char*)buf, nullptr);
    return ICS_OK;
  });
}

int ics_load_checkpoint(ics_handle hh, const void* buf, int64_t bytes) {
  if (!hh || !buf || bytes < (int64_t)sizeof(CkptHeader)) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    if (h.cases.n) {
      h.err = "checkpoints do not carry the per-case controls of stacked cases";
      return ICS_ERR_ARG;
    }
    CkptHeader hd;
    std::memcpy(&hd, buf, sizeof(hd));
    const CkptHeader mine = ckpt_header(h);
    if (std::memcmp(hd.magic, mine.magic, 8) != 0 || hd.version != CKPT_VERSION || hd.N != mine.N ||
        hd.F != mine.F || hd.B != mine.B || hd.nInst != mine.nInst || hd.scalarOn != mine.scalarOn) {
      h.err = "checkpoint does not match this handle (mesh, instances or scalar transport)";
      return ICS_ERR_ARG;
    }
    int64_t need = 0;
    ics_checkpoint_size(hh, &need);
    if (bytes < need) {
      h.err = "checkpoint truncated";
      return ICS_ERR_ARG;
    }
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    CkptHeader tmp = hd;
    ckpt_walk(h, tmp, nullptr, (const char*)buf);
    h.timeIndex = hd.timeIndex;
    h.initResValid = hd.initResValid != 0;
    h.prevResValid = hd.prevResValid != 0;
    h.lastRhoL2 = hd.lastRhoL2;
    h.haveFlux = h.haveMatrix = h.haveIncrement = h.haveExact = false;
    return ICS_OK;
  });
}

// passive scalar transport ---------------------------------------------------
__global__ void k_scalar_init(int N, const double* __restrict__ s, const double* __restrict__ W,
                              double* __restrict__ rhoS) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < N) rhoS[c] = W[5 * c] * s[c];
}

int ics_scalar_enable(ics_handle hh, const double* s, const int32_t* patch_fixed, const double* patch_value,
                      double D, int32_t recon) {
  if (!hh || !s || recon < 0 || recon > ICS_RECON_MUSCL_MINMOD || !(D >= 0)) return ICS_ERR_ARG;
  if (hh->h.m.nInst > 1) {
    hh->h.err = "scalar transport is not provided for Harmonic Balance handles";
    return ICS_ERR_ARG;
  }
  if (hh->h.cases.n) {
    hh->h.err = "stacked cases carry no passive scalar";
    return ICS_ERR_ARG;
  }
  if (hh->h.m.ncyc > 0 && hh->h.cfg.c.viscous) {
    hh->h.err = "the scalar's laplacian across cyclic patches is not built";
    return ICS_ERR_ARG;
  }
  return guard(hh, [&](Handle& h) {
    const size_t N = h.m.N, F = h.m.F, B = h.m.B, P = h.m.npatches;
    if (!h.ss) {
      h.ss = dalloc<double>(N);
      h.ssB = dalloc<double>(B);
      h.srhoS = dalloc<double>(N);
      h.srhoS0 = dalloc<double>(N);
      h.srhoS00 = dalloc<double>(N);
      h.sgrad = dalloc<double>(3 * N);
      h.sgradL = dalloc<double>(3 * N);
      h.sface = dalloc<double>(5 * (F + B));
      h.sblk = dalloc<double>((size_t)h.m.nslots * 32);
      h.sdg = dalloc<double>(N);
      h.srD = dalloc<double>(N);
      h.ssrc = dalloc<double>(N);
      h.sFixed = dalloc<int>(P ? P : 1);
      h.sValue = dalloc<double>(P ? P : 1);
    }
    std::vector<int> fx(P, 0);
    std::vector<double> val(P, 0.0);
    for (size_t p = 0; p < P; ++p) {
      fx[p] = patch_fixed ? (patch_fixed[p] != 0) : 0;
      val[p] = patch_value ? patch_value[p] : 0.0;
    }
    if (P) {
      ICS_CUDA(cudaMemcpy(h.sFixed, fx.data(), P * sizeof(int), cudaMemcpyHostToDevice));
      ICS_CUDA(cudaMemcpy(h.sValue, val.data(), P * sizeof(double), cudaMemcpyHostToDevice));
    }
    ICS_CUDA(cudaMemcpyAsync(h.ss, s, N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    k_scalar_init<<<grid_for(N, 256), 256, 0, h.stream>>>((int)N, h.ss, h.W, h.srhoS);
    ICS_CUDA(cudaGetLastError());
    h.launches++;
    ICS_CUDA(cudaMemcpyAsync(h.srhoS0, h.srhoS, N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
    ICS_CUDA(cudaMemcpyAsync(h.srhoS00, h.srhoS, N * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
    h.Ds = D;
    h.reconS = recon;
    h.scalarOn = true;
    launch_scalar_bc(h);
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    return ICS_OK;
  });
}

int ics_scalar_transport(ics_handle hh, int32_t n_iterations, ics_solver_perf* perf) {
  if (!hh || n_iterations < 0) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    if (!h.scalarOn) {
      h.err = "scalar transport is not enabled";
      return ICS_ERR_STATE;
    }
    ensure_workspace(h);
    Range rg("ics scalar transport");
    ics_solver_perf pf;
    std::memset(&pf, 0, sizeof(pf));
    double* dx = (double*)h.kx;
    for (int it = 0; it < n_iterations; ++it) {
      ICS_CUDA(cudaMemsetAsync(&h.ks->status, 0, sizeof(int), h.stream));
      launch_scalar_assembly(h);
      int stt = 0;
      ICS_CUDA(cudaMemcpyAsync(&stt, &h.ks->status, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
      ICS_CUDA(cudaStreamSynchronize(h.stream));
      if (stt) {
        h.err = "All diagonals of the scalar matrix are zero";
        return ICS_ERR_DIAG;
      }
      const int st = scalar_gmres(h, dx, &pf);
      if (st && st != ICS_ERR_BREAKDOWN) {
        h.err = "non-finite scalar Krylov residual";
        return st;
      }
      launch_scalar_update(h, dx);
    }
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (perf) *perf = pf;
    return ICS_OK;
  });
}

int ics_get_scalar(ics_handle hh, double* s, double* rhoS) {
  return guard(hh, [&](Handle& h) {
    if (!h.scalarOn) return ICS_ERR_STATE;
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (s) ICS_CUDA(cudaMemcpy(s, h.ss, h.m.N * sizeof(double), cudaMemcpyDeviceToHost));
    if (rhoS) ICS_CUDA(cudaMemcpy(rhoS, h.srhoS, h.m.N * sizeof(double), cudaMemcpyDeviceToHost));
    return ICS_OK;
  });
}

// Jacobian-vector products of the residual source ------------------------
namespace {
void ensure_tangent(Handle& h) {
  if (h.tW) return;
  const size_t N = h.m.N, FB = (size_t)h.m.F + h.m.B, D = 2 * sizeof(double);
  auto dal = [&](size_t bytes) {
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) throw CudaError(e, "cudaMalloc", __FILE__, __LINE__);
    return p;
  };
  h.tW = dal(5 * N * D);
  h.tprim = dal(5 * N * D);
  h.tq = dal(NQ * N * D);
  h.tgrad = dal(3 * NQ * N * D);
  h.tflux = dal(5 * FB * D);
  h.tvc = dal(24 * N * D);
  h.tfv = dal(8 * FB * D);
  h.tv = (double*)dal(10 * N * sizeof(double));
}

// stage a [N][5] input into dst (device) from a host or device pointer
void stage_in(Handle& h, const double* src, double* dst, int device) {
  ICS_CUDA(cudaMemcpyAsync(dst, src, 5ull * h.m.N * sizeof(double),
                           device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h.stream));
}
void stage_out(Handle& h, const double* src, double* dst, int device) {
  ICS_CUDA(cudaMemcpyAsync(dst, src, 5ull * h.m.N * sizeof(double),
                           device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h.stream));
  ICS_CUDA(cudaStreamSynchronize(h.stream));
}
}  // namespace

int ics_jvp(ics_handle hh, const double* v, double* Jv, int32_t device) {
  if (!v || !Jv) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    ensure_tangent(h);
    Range rg("ics jvp");
    double* tv = h.tv;
    double* out = h.tv + 5ull * h.m.N;
    stage_in(h, v, tv, device);
    launch_residual_tangent(h, tv, out);
    stage_out(h, out, Jv, device);
    return ICS_OK;
  });
}

int ics_assemble_exact_jacobian(ics_handle hh, int64_t* nnz_blocks, int32_t* n_colours) {
  return guard(hh, [&](Handle& h) {
    ensure_tangent(h);
    assemble_exact(h);
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (nnz_blocks) *nnz_blocks = h.xnnz;
    if (n_colours) *n_colours = h.xncol;
    return ICS_OK;
  });
}

int ics_get_exact_jacobian(ics_handle hh, int32_t* row_ptr, int32_t* cols, double* blocks) {
  return guard(hh, [&](Handle& h) {
    if (!h.haveExact) {
      h.err = "get_exact_jacobian needs ics_assemble_exact_jacobian at the current state";
      return ICS_ERR_STATE;
    }
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (row_ptr) ICS_CUDA(cudaMemcpy(row_ptr, h.xptr, (h.m.N + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    if (cols) ICS_CUDA(cudaMemcpy(cols, h.xcol, h.xnnz * sizeof(int), cudaMemcpyDeviceToHost));
    if (blocks) ICS_CUDA(cudaMemcpy(blocks, h.xblk, h.xnnz * 25 * sizeof(double), cudaMemcpyDeviceToHost));
    return ICS_OK;
  });
}

int ics_vjp(ics_handle hh, const double* u, double* JTu, int32_t device) {
  if (!u || !JTu) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    ensure_tangent(h);
    Range rg("ics vjp");
    if (!h.haveExact) assemble_exact(h);
    double* tu = h.tv;
    double* out = h.tv + 5ull * h.m.N;
    stage_in(h, u, tu, device);
    exact_vjp(h, tu, out);
    stage_out(h, out, JTu, device);
    return ICS_OK;
  });
}

namespace {
// autotuner choices per (device, cells, faces, slots, levels, precision, scheme, limiter)
std::mutex g_tune_mu;
std::map<std::vector<long long>, ics_tuning> g_tune_cache;
std::vector<long long> tune_key(const Handle& h) {
  int lim = 0;
  grad_mask(h, &lim);
  return {h.device, h.m.N, h.m.F, h.m.nslots, h.m.nfl, h.m.nrl, prec(h), h.cfg.c.flux_scheme, lim,
          h.cfg.c.preconditioner, h.cfg.c.n_directions};
}
}  // namespace

int ics_autotune(ics_handle hh, ics_tuning* out) {
  return guard(hh, [&](Handle& h) {
    if (!h.haveMatrix || !h.haveFlux) {
      h.err = "autotune needs a residual and an assembled Jacobian";
      return ICS_ERR_STATE;
    }
    const auto key = tune_key(h);
    ics_tuning t{};
    {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) t = it->second, t.from_cache = 1;
    }
    if (!t.from_cache) {
      std::vector<std::pair<std::string, double>> log;
      autotune_residual(h, log);
      autotune_linalg(h, log);
      t.face_block = h.tuneFaceBs;
      t.grad_block = h.tuneGradBs;
      t.mgs_blocks = h.tuneMgsBlocks;
      t.fused_operator = h.tuneFused;
      t.reverse_rows = h.tuneRevRows;
      std::lock_guard<std::mutex> lock(g_tune_mu);
      g_tune_cache[key] = t;
    }
    h.tuneFaceBs = t.face_block;
    h.tuneGradBs = t.grad_block;
    h.tuneMgsBlocks = t.mgs_blocks;
    h.tuneFused = t.fused_operator;
    h.tuneRevRows = t.reverse_rows;
    drop_graphs(h);  // the captured cycle holds the old launch shapes
    // the timing runs overwrote the Krylov workspace and the face fields
    // of this state; the next iteration recomputes both
    h.haveIncrement = false;
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (out) *out = t;
    return ICS_OK;
  });
}

int ics_set_tuning(ics_handle hh, const ics_tuning* t) {
  if (!t) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    const bool ok = (t->face_block == 64 || t->face_block == 128) && (t->grad_block == 64 || t->grad_block == 128) &&
                    (t->mgs_blocks == 152 || t->mgs_blocks == 304 || t->mgs_blocks == 456 || t->mgs_blocks == 608) &&
                    (t->fused_operator == 0 || t->fused_operator == 1) &&
                    (t->reverse_rows == 1 || t->reverse_rows == 2);
    if (!ok) {
      h.err = "tuning values outside the autotuner's candidates";
      return ICS_ERR_ARG;
    }
    h.tuneFaceBs = t->face_block;
    h.tuneGradBs = t->grad_block;
    h.tuneMgsBlocks = t->mgs_blocks;
    h.tuneFused = t->fused_operator;
    h.tuneRevRows = t->reverse_rows;
    drop_graphs(h);
    return ICS_OK;
  });
}

int ics_vjp_recompute(ics_handle hh, const double* u, double* JTu, int32_t device) {
  if (!u || !JTu) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    const std::string why = residual_vjp_unsupported(h);
    if (!why.empty()) {
      h.err = why;
      return ICS_ERR_ARG;
    }
    ensure_tangent(h);
    Range rg("ics vjp_recompute");
    double* tu = h.tv;
    double* out = h.tv + 5ull * h.m.N;
    stage_in(h, u, tu, device);
    launch_residual_vjp(h, tu, out);
    stage_out(h, out, JTu, device);
    return ICS_OK;
  });
}

namespace {
// one matrix-free Krylov solve with host right-hand side and solution
using KrylovSolve = int (*)(Handle&, const double*, double*, const ics_krylov_opts&, ics_krylov_result*);
int krylov_entry(ics_handle hh, const double* rhs, double* sol, const ics_krylov_opts* opts,
                 ics_krylov_result* result, KrylovSolve solve, const char* name) {
  if (!rhs || !sol || !opts) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    ensure_tangent(h);
    Range rg(name);
    double* d = h.tv;
    double* x = h.tv + 5ull * h.m.N;
    stage_in(h, rhs, d, 0);
    ics_krylov_result r{};
    const int st = solve(h, d, x, *opts, &r);
    if (result) *result = r;
    stage_out(h, x, sol, 0);
    return st;
  });
}
}  // namespace

int ics_adjoint_solve(ics_handle hh, const double* g, double* psi, const ics_krylov_opts* opts,
                      ics_krylov_result* result) {
  return krylov_entry(hh, g, psi, opts, result, adjoint_solve, "ics adjoint_solve");
}

int ics_tangent_solve(ics_handle hh, const double* b, double* x, const ics_krylov_opts* opts,
                      ics_krylov_result* result) {
  return krylov_entry(hh, b, x, opts, result, tangent_solve, "ics tangent_solve");
}

int ics_pressure_force(ics_handle hh, int32_t patch, const double dir[3], double* J, double* dJdW) {
  if (!dir || !J) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    if (patch < 0 || patch >= h.m.npatches) {
      h.err = "pressure_force: no such patch";
      return ICS_ERR_ARG;
    }
    std::vector<Patch> ps(h.m.npatches);
    ICS_CUDA(cudaMemcpy(ps.data(), h.m.patches, ps.size() * sizeof(Patch), cudaMemcpyDeviceToHost));
    const int k = ps[patch].kind;
    if (k != ICS_PATCH_SLIP && k != ICS_PATCH_ZERO_GRADIENT && k != ICS_PATCH_ISOTHERMAL_WALL) {
      h.err = "pressure_force: the patch's pressure is not zeroGradient";
      return ICS_ERR_ARG;
    }
    ensure_tangent(h);
    double* d = dJdW ? h.tv : nullptr;
    *J = pressure_force(h, patch, dir, d);
    if (dJdW) stage_out(h, d, dJdW, 0);
    return ICS_OK;
  });
}

int ics_pseudo_loop(ics_handle hh, int32_t* more) {
  if (!more) return ICS_ERR_ARG;
  return guard(hh, [&](Handle& h) {
    // every instance's control advances (no short cut); more while any runs
    bool any = false;
    if (h.cases.n) {
      // stacked cases: a case whose loop completes stays frozen until all have
      CaseSet& S = h.cases;
      for (int k = 0; k < S.n; ++k) {
        if (S.frozen[k]) continue;
        if (pseudo_loop_one(h, S.ctl[k]))
          any = true;
        else
          S.frozen[k] = 1;
      }
      if (!any) std::fill(S.frozen.begin(), S.frozen.end(), 0);
      *more = any ? 1 : 0;
      return ICS_OK;
    }
    for (auto& q : h.ctl) any = pseudo_loop_one(h, q) || any;
    *more = any ? 1 : 0;
    return ICS_OK;
  });
}

int ics_set_hb(ics_handle hh, int32_t n, const double* D) {
  if (!hh) return ICS_ERR_ARG;
  Handle& h0 = hh->h;
  if (n < 1 || n > MAX_INST || (n > 1 && !D)) {
    h0.err = "n_instances must be in [1, ICS_MAX_INSTANCES] with an operator";
    return ICS_ERR_ARG;
  }
  if (h0.m.N % n != 0) {
    h0.err = "cell count is not a multiple of the number of instances";
    return ICS_ERR_ARG;
  }
  if (n > 1 && h0.cases.n) {
    h0.err = "stacked cases are not combined with Harmonic Balance";
    return ICS_ERR_ARG;
  }
  if (n > 1 && (h0.cfg.c.ddt_scheme != ICS_DDT_STEADY || h0.cfg.c.solver != ICS_SOLVER_GMRES)) {
    h0.err = "Harmonic Balance needs steadyState ddt and the GMRES solver";
    return ICS_ERR_ARG;
  }
  for (int q = 0; n > 1 && q < n * n; ++q)
    if (!std::isfinite(D[q])) {
      h0.err = "non-finite Harmonic Balance operator";
      return ICS_ERR_ARG;
    }
  return guard(hh, [&](Handle& h) {
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (h.m.Dhb) ICS_CUDA(cudaFree(h.m.Dhb));
    h.m.Dhb = nullptr;
    if (n > 1) {
      h.m.Dhb = dalloc<double>((size_t)n * n);
      ICS_CUDA(cudaMemcpy(h.m.Dhb, D, sizeof(double) * n * n, cudaMemcpyHostToDevice));
    }
    h.m.nInst = n;
    h.m.Nc = h.m.N / n;
    // a new instance count starts without a zone (every cell) and Cartesian
    if (h.hbZoneBuf) ICS_CUDA(cudaFree(h.hbZoneBuf));
    h.hbZoneBuf = nullptr;
    h.m.hbZone = nullptr;
    h.m.hbCyl = 0;
    h.ctl.assign(n, Handle::Control());
    h.initResValid = h.prevResValid = false;
    h.haveMatrix = h.haveIncrement = false;
    free_exact(h);   // the stencil gains the instance partners
    drop_graphs(h);  // the captured cycle's reduction grids depend on n
    return ICS_OK;
  });
}

int ics_set_hb_zone(ics_handle hh, const int32_t* zone, int32_t cyl_coords, const double axis[3],
                    const double origin[3]) {
  if (!hh) return ICS_ERR_ARG;
  Handle& h0 = hh->h;
  if (h0.m.nInst < 2) {
    h0.err = "set_hb_zone needs a Harmonic Balance handle";
    return ICS_ERR_ARG;
  }
  double a[3] = {0, 0, 1}, o[3] = {0, 0, 0};
  if (cyl_coords) {
    if (!axis || !origin) {
      h0.err = "cylCoords needs the rotation axis and origin";
      return ICS_ERR_ARG;
    }
    const double ma = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
    if (!(ma > 0)) {
      h0.err = "zero rotation axis";
      return ICS_ERR_ARG;
    }
    for (int k = 0; k < 3; ++k) {
      a[k] = axis[k] / ma;
      o[k] = origin[k];
    }
  }
  return guard(hh, [&](Handle& h) {
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    if (h.hbZoneBuf) ICS_CUDA(cudaFree(h.hbZoneBuf));
    h.hbZoneBuf = nullptr;
    h.m.hbZone = nullptr;
    if (zone) {
      std::vector<unsigned char> mask(h.m.N);
      for (int c = 0; c < h.m.N; ++c) mask[c] = zone[c % h.m.Nc] != 0;
      h.hbZoneBuf = dalloc<unsigned char>(h.m.N);
      ICS_CUDA(cudaMemcpy(h.hbZoneBuf, mask.data(), h.m.N, cudaMemcpyHostToDevice));
      h.m.hbZone = h.hbZoneBuf;
    }
    h.m.hbCyl = cyl_coords ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
      h.m.hbAxis[k] = a[k];
      h.m.hbOrigin[k] = o[k];
    }
    h.haveMatrix = h.haveIncrement = h.haveExact = false;
    drop_graphs(h);  // the captured launches hold DevMesh by value
    return ICS_OK;
  });
}

int ics_set_phase_lag(ics_handle hh, const int32_t* mode, const double* P) {
  if (!hh) return ICS_ERR_ARG;
  Handle& h0 = hh->h;
  const int np = h0.m.npatches, n = h0.m.nInst;
  if (mode) {
    if (n < 2 || !P) {
      h0.err = "phase lag needs a Harmonic Balance handle and the operators";
      return ICS_ERR_ARG;
    }
  }
  return guard(hh, [&](Handle& h) {
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    std::vector<Patch> pts(np);
    if (np) ICS_CUDA(cudaMemcpy(pts.data(), h.m.patches, np * sizeof(Patch), cudaMemcpyDeviceToHost));
    if (mode)
      for (int p = 0; p < np; ++p)
        if (mode[p] < 0 || mode[p] > 2 || (mode[p] && pts[p].kind != ICS_PATCH_CYCLIC))
          throw std::string("phase-lag modes must be 0, 1 or 2 and set on cyclic patches only");
    dfree(h.m.plagMode);
    dfree(h.m.plagP);
    h.m.plagMode = nullptr;
    h.m.plagP = nullptr;
    h.haveFlux = h.haveMatrix = h.haveIncrement = false;
    free_exact(h);  // the stencil gains the other instances' partners
    drop_graphs(h);
    if (!mode) return ICS_OK;
    h.m.plagMode = upload(std::vector<int>(mode, mode + np));
    h.m.plagP = upload(std::vector<double>(P, P + (size_t)np * n * n));
    return ICS_OK;
  });
}

int ics_set_mrf(ics_handle hh, const double* omega, const double* face_velocity, const double* boundary_U,
                const int32_t* included, int32_t mode) {
  if (!hh) return ICS_ERR_ARG;
  Handle& h0 = hh->h;
  const int N = h0.m.N, F = h0.m.F, B = h0.m.B;
  if (omega) {
    if (!face_velocity || (B > 0 && (!boundary_U || !included)) ||
        (mode != ICS_MRF_OUTER_LOOP && mode != ICS_MRF_EVERY_UPDATE)) {
      h0.err = "MRF zones need omega, face_velocity, boundary_U, included and a known mode";
      return ICS_ERR_ARG;
    }
    bool ok = true;
    for (long i = 0; i < 3L * N && ok; ++i) ok = std::isfinite(omega[i]);
    for (long i = 0; i < (long)F + B && ok; ++i) ok = std::isfinite(face_velocity[i]);
    for (long i = 0; i < 3L * B && ok; ++i) ok = std::isfinite(boundary_U[i]);
    for (long i = 0; i < B && ok; ++i) ok = included[i] == 0 || included[i] == 1;
    if (!ok) {
      h0.err = "non-finite MRF field or an included flag other than 0/1";
      return ICS_ERR_ARG;
    }
  }
  return guard(hh, [&](Handle& h) {
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    DevMesh& m = h.m;
    void* old[] = {m.mrfU, m.mrfOm, m.mrfBU, m.mrfBIn};
    for (void* p : old) dfree(p);
    m.mrfU = m.mrfOm = m.mrfBU = nullptr;
    m.mrfBIn = nullptr;
    m.mrfEvery = 0;
    h.haveExact = false;
    h.haveFlux = h.haveMatrix = h.haveIncrement = false;
    drop_graphs(h);
    if (!omega) return ICS_OK;
    std::vector<double> om(3ull * N), bu(3ull * B);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < 3; ++k) om[(size_t)k * N + i] = omega[3 * i + k];
    for (int b = 0; b < B; ++b)
      for (int k = 0; k < 3; ++k) bu[(size_t)k * B + b] = boundary_U[3 * b + k];
    m.mrfOm = upload(om);
    m.mrfU = upload(std::vector<double>(face_velocity, face_velocity + F + B));
    if (B > 0) {
      m.mrfBU = upload(bu);
      m.mrfBIn = upload(std::vector<int>(included, included + B));
    }
    m.mrfEvery = mode == ICS_MRF_EVERY_UPDATE;
    // createFields.H:262-263: the boundary velocity is assigned at once
    launch_mrf_bc(h);
    ICS_CUDA(cudaStreamSynchronize(h.stream));
    return ICS_OK;
  });
}

}  // extern "C"
