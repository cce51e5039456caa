// Internal declarations of the GB300 hot path.
//
// Device data layout (all resident for the life of a handle):
//   * cell 5-vectors  [N][5]  AoS (rho, rhoUx, rhoUy, rhoUz, rhoE): one
//     gather of a neighbour's state is one 40-byte (FP64) or 20-byte (FP32)
//     contiguous read.
//   * reconstructed scalars and their gradients: SoA [k][N] and [k][3][N],
//     coalesced for the cell- and face-parallel kernels.
//   * face arrays: SoA [F] per component, face-parallel kernels read them
//     with unit stride.
//   * Jacobian: sliced-ELL with slice height 32 (one warp) of 5x5 blocks.
//     Row = cell, one slot per internal face of that cell, slots sorted by
//     column (lower part first).  Block entry k of slot t of slice s for lane
//     l lives at ((slot_base[s] + t) * 25 + k) * 32 + l, so a warp reading
//     one entry of its 32 rows touches one contiguous 256 B (FP64) line.
//     The diagonal block of cell c lives at ((c/32) * 25 + k) * 32 + c%32.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "icsfoam_gb300.h"

namespace ics {

constexpr double SMALL = 1e-15;
constexpr double VSMALL = 1e-300;
constexpr double ROOTVSMALL = 1e-150;
constexpr double GREAT = 1e15;
constexpr double VGREAT = 1e300;

// reconstructed scalar fields (slots of q[][N])
enum { Q_RHO = 0, Q_P = 1, Q_UX = 2, Q_UY = 3, Q_UZ = 4, Q_E = 5, Q_H = 6, Q_C = 7, NQ = 8 };

constexpr int SLICE = 32;
constexpr int REDUCE_BLOCKS = 1216;  // 8 x 152 SMs
constexpr int MAX_DIRS = 64;
constexpr int MAX_INST = ICS_MAX_INSTANCES;  // Harmonic Balance instances

// Scalars living in device memory for the Krylov cycle (one per handle).
struct KrylovScalars {
  double H[MAX_DIRS * MAX_DIRS];
  double c[MAX_DIRS], s[MAX_DIRS], bh[MAX_DIRS + 1], y[MAX_DIRS];
  double beta;            // norm used to scale the next Krylov vector
  double red[16];         // reduction results
  double avg[5 * MAX_INST];  // per-instance field averages of W
  double nfr[8 * MAX_INST];  // per instance: norm-factor sums (rho, rhoE, rhoU), |b| per equation
  double res[5 * MAX_INST];  // per-instance L1 residuals (unnormalised sums)
  double l2;              // rho L2 partial result
  int status;             // breakdown / non-finite flags
};

struct Patch {
  int kind, is_wall;
  double p, T, U[3], p0, T0;
  double R[9];  // cyclic: partner-side vectors into this patch's frame
};

struct DevMesh {
  int N = 0, F = 0, B = 0, nslices = 0, nslots = 0;
  int solD[3] = {1, 1, 1};
  int* own = nullptr;
  int* nei = nullptr;
  double* Sf = nullptr;      // [3][F] SoA
  double* magSf = nullptr;   // [F]
  double* w = nullptr;       // [F]
  double* nodc = nullptr;    // [F]
  double* dc = nullptr;      // [F] deltaCoeffs 1/|C_nei - C_own|
  double* dOwn = nullptr;    // [3][F] Cf - C[own]
  double* dNei = nullptr;    // [3][F] Cf - C[nei]
  double* dCC = nullptr;     // [3][F] C[nei] - C[own]
  double* nf = nullptr;      // [3][F] Sf/magSf
  double* bnf = nullptr;     // [3][B] Sf/magSf
  double* C = nullptr;       // [3][N]
  double* V = nullptr;       // [N]
  int* bcell = nullptr;      // [B]
  int* bpatch = nullptr;     // [B]
  double* bSf = nullptr;     // [3][B]
  double* bmagSf = nullptr;  // [B]
  double* bdOwn = nullptr;   // [3][B] Cf - C
  double* bdc = nullptr;     // [B]
  Patch* patches = nullptr;
  int npatches = 0;
  // cell -> internal faces CSR in increasing face order (code f: owner side, ~f: neighbour side)
  int* cptr = nullptr;
  int* cface = nullptr;
  // cell -> boundary faces CSR
  int* bptr = nullptr;
  int* bface = nullptr;
  // sliced-ELL structure
  int* slot_base = nullptr;  // [nslices+1]
  int* scol = nullptr;       // [nslots*32] column or -1
  int* sface = nullptr;      // [nslots*32] face code or 0x7fffffff
  int* nlow = nullptr;       // [N] number of lower slots
  int* nslot = nullptr;      // [N] number of slots
  // LU-SGS level schedule
  int nfl = 0, nrl = 0;              // number of forward / reverse levels
  std::vector<int> fl_ptr, rl_ptr;   // host copies of level pointers
  std::vector<int> fl_cstart, rl_cstart;  // first cell when a level is a contiguous range, else -1
  int* fl_cells = nullptr;           // cells by forward level
  int* rl_cells = nullptr;           // cells by reverse level
  int* fl_lptr = nullptr;            // device copies of the level pointers
  int* rl_lptr = nullptr;
  void* sweep_pad = nullptr;         // [2][8N] FP64-sized outputs of the sync-free sweeps
  unsigned int* sweep_ticket = nullptr;  // [2] row tickets of the sync-free sweeps
  bool fuse_last = false;            // last forward level == first reverse level (same rows)
  // Harmonic Balance: nInst stacked instances of Nc cells (instance-major),
  // coupled through the spectral operator Dhb [nInst][nInst]
  int nInst = 1, Nc = 0;
  double* Dhb = nullptr;
  // HB zone (HBZone cellZone): cells of the stacked mesh that carry the
  // spectral source and couplings (nullptr: every cell); hbCyl combines the
  // instances' momentum in cylindrical components about hbAxis through
  // hbOrigin (HBZone cylCoords)
  const unsigned char* hbZone = nullptr;
  int hbCyl = 0;
  double hbAxis[3] = {0, 0, 1}, hbOrigin[3] = {0, 0, 0};
  // moving reference frames (all nullptr without MRF zones): frame velocity
  // . n per internal then boundary face [F+B], rotation vector per cell
  // [3][N], frame velocity of the boundary faces [3][B] and where it is
  // assigned [B]; mrfEvery re-assigns it after every boundary update
  // coupled (cyclic) boundary faces: partner cell [B] (-1 elsewhere),
  // weights [B], delta (partner centre seen from this side minus C) [3][B],
  // partner-side displacement Cf - C - delta [3][B], nonOrthDeltaCoeffs [B];
  // the cyclic faces grouped by cell (cyc_face, in increasing cell order) and
  // the rows that own them (cyc_row with cyc_ptr into cyc_face)
  int* bpartner = nullptr;
  double* bw = nullptr;
  double* bdelta = nullptr;
  double* bdNei = nullptr;
  double* bnodc = nullptr;
  int ncyc = 0, ncrow = 0;
  int* cyc_face = nullptr;
  int* cyc_row = nullptr;
  int* cyc_ptr = nullptr;
  // phase-lag cyclic patches (Harmonic Balance): per patch 0 plain, 1 phase
  // lag, 2 phase lag with cylindrical velocity; per patch the instances'
  // operator P [npatches][nInst][nInst]
  int* plagMode = nullptr;
  double* plagP = nullptr;
  // ratio of specific heats (the phase-lagged sound speed, the factored
  // off-diagonal blocks)
  double gamma = 1.4;
  // cellLimited coefficient k as the widening factor 1/k - 1 of the bounds
  double limWiden = 0.0;
  // non-LF viscous parts of the off-diagonal blocks (blocks.cuh), block
  // storage type; nullptr unless that Jacobian mode is assembled
  const void* vjslot = nullptr;
  const void* vjcell = nullptr;
  double* mrfU = nullptr;
  double* mrfOm = nullptr;
  double* mrfBU = nullptr;
  int* mrfBIn = nullptr;
  int mrfEvery = 0;
  // independent cases stacked in one mesh (nullptr otherwise): case of each
  // cell [N] and each case's SER factor [n_cases] (< 0: not applied)
  const int* caseOf = nullptr;
  const double* caseSer = nullptr;
  // and each case's Krylov norm and flags (the fused operator's scaling)
  const double* caseBeta = nullptr;
  const int* caseActive = nullptr;
  const int* caseStatus = nullptr;
};

// pseudotimeControl state (pseudotimeControl.C): the iteration count of the
// current time step, convergence flags and the last / first residuals
struct PseudoControl {
  int corr = 0;
  bool converged = false, firstIteration = true;
  double residuals[5] = {0, 0, 0, 0, 0}, initResiduals[5] = {0, 0, 0, 0, 0};
};

// Device view of the stacked cases' per-case state (ics_set_cases): the
// reduction segments (block b reduces cells segBeg[b] .. segEnd[b]-1 of case
// segCase[b]; case k owns segments caseSeg[k] .. caseSeg[k+1]-1), and per
// case its Krylov scalars with a Hessenberg of m x m.
struct CaseDev {
  int n = 0, m = 0;
  const int* segCase = nullptr;
  const int* segBeg = nullptr;
  const int* segEnd = nullptr;
  const int* caseSeg = nullptr;
  const int* start = nullptr;     // [n+1] cells
  const int* active = nullptr;    // [n] 1: the case takes part in this solve
  double* partials = nullptr;     // [nseg][8]
  unsigned int* counter = nullptr;  // [n]
  double* H = nullptr;            // [n][m*m]
  double* c = nullptr;            // [n][m]
  double* s = nullptr;            // [n][m]
  double* bh = nullptr;           // [n][m+1]
  double* y = nullptr;            // [n][m]
  double* beta = nullptr;         // [n]
  double* red = nullptr;          // [n][2]
  double* res = nullptr;          // [n][5] L1 residual sums
  double* nfr = nullptr;          // [n][8] norm-factor and |b| sums
  double* avg = nullptr;          // [n][5] averages of W
  double* l2 = nullptr;           // [n] sums of (R_rho V)^2
  int* status = nullptr;          // [n] breakdown / non-finite flags
};

struct CaseSet {
  int n = 0, nseg = 0;
  std::vector<int> start;          // host [n+1]
  CaseDev d;
  int* caseOf = nullptr;           // device [N]
  double* ser = nullptr;           // device [n]
  void* mem = nullptr;             // one device allocation behind d's arrays
  // pinned host mirrors of res, nfr, l2, status, active
  double* hres = nullptr;
  double* hnfr = nullptr;
  double* hl2 = nullptr;
  int* hstatus = nullptr;
  int* hactive = nullptr;
  double* hser = nullptr;
  // host bookkeeping per case (what a handle of its own keeps)
  std::vector<PseudoControl> ctl;
  std::vector<double> initRes, prevRes, finRes;  // [5n]
  std::vector<char> initValid, prevValid, frozen;
  std::vector<int> cycles;
};

struct Cfg {
  ics_config c;
  double Cv, gamma;
};

struct Handle {
  DevMesh m;
  Cfg cfg;
  cudaStream_t stream = nullptr;
  int device = 0;  // the CUDA device current at ics_create (owns the stream and every buffer)
  std::string err;
  // state
  double* W = nullptr;      // [N][5]
  double* W0 = nullptr;
  double* W00 = nullptr;
  double* Wprev = nullptr;
  double* prim = nullptr;   // [5][N]: p, T, Ux, Uy, Uz
  double* pB = nullptr;     // [B]
  double* TB = nullptr;
  double* UB = nullptr;     // [3][B]
  double* phiB = nullptr;
  double* pseudoCo = nullptr;
  double* rPDT = nullptr;
  double* ddtCoeff = nullptr;
  int timeIndex = 0;
  // residual pipeline
  double* q = nullptr;      // [NQ][N]
  double* bq = nullptr;     // [NQ][B]
  double* clin = nullptr;   // [N] sqrt(gamma/psi)
  double* grad = nullptr;   // [NQ][3][N]
  double* fflux = nullptr;  // [5][F+B]
  double* frec = nullptr;   // [8][F]: ULx,ULy,ULz,URx,URy,URz,EL,ER
  double* flam = nullptr;   // [F+B]
  double* cfrec = nullptr;  // [8][ncyc]: the reconstructed states of the cyclic faces (as frec)
  void* cblk = nullptr;     // [ncyc][25] cyclic coupling blocks (partner rotation folded in)
  void* vjslotbuf = nullptr;  // non-LF viscous block parts (FP64-sized): [nslots][2][32]
  void* vjcellbuf = nullptr;  // and [5][N]
  double* bjac = nullptr;   // [25][B] boundary Jacobian diag contribution
  double* src = nullptr;    // [N][5] source = R*V
  // viscous terms (allocated when the case is viscous)
  double* vcell = nullptr;  // [24][N] grad U, grad e, tauMC, mu, alphaEff, e
  double* fvisc = nullptr;  // [8][F+B] lapU, divTau, divSig, lapE face terms
  double* vsf2 = nullptr;   // [F] LF viscous Jacobian coefficient
  double* vjac = nullptr;   // [2][F+B] non-LF viscous laplacian coefficients: internal and
                            // coupled faces (mu_f|S|) dc, (alpha_f|S|) dc; boundary mu_b, alpha_b
  // Jacobian (FP64 or FP32 storage by precision)
  void* blk = nullptr;      // [nslots*25*32]
  void* dg = nullptr;       // [nslices*25*32]
  void* dginv = nullptr;    // Jacobi inverse, same layout as dg
  void* rD = nullptr;       // [N]
  bool haveMatrix = false, haveIncrement = false, haveFlux = false;
  int jacPrecision = ICS_PREC_FP64;
  // Krylov workspace (element type by precision)
  void* kv = nullptr;       // [m][N][5]
  void* kw = nullptr;       // [N][5]
  void* kx = nullptr;       // [N][5]
  void* kb = nullptr;       // [N][5]
  void* kt = nullptr;       // [N][5]
  double* dW = nullptr;     // [N][5]
  int kvDirs = 0, kvPrec = -1;
  // reductions
  double* partials = nullptr;   // [REDUCE_BLOCKS * 16]
  unsigned int* counter = nullptr;
  KrylovScalars* ks = nullptr;  // device
  KrylovScalars* ksHost = nullptr;  // pinned mirror
  // host-side residual bookkeeping (setCoAndDeltaT.H, pseudotimeControl):
  // linear-solver initial residuals per instance and equation, [5*J + k]
  bool initResValid = false, prevResValid = false;
  std::vector<double> initRes, prevRes;
  // one pseudotimeControl per instance (the HB solver loops while any runs)
  using Control = PseudoControl;
  std::vector<Control> ctl = std::vector<Control>(1);
  double lastRhoL2 = 0;
  // residual tangent (Jacobian-vector product) workspace of dual numbers
  // (value, derivative), allocated on first use: W, prim [5N], q [NQ N],
  // grad [3 NQ N], face fluxes [5 (F+B)], viscous cell terms [24 N] and
  // viscous face terms [8 (F+B)]
  void* tW = nullptr;
  void* tprim = nullptr;
  void* tq = nullptr;
  void* tgrad = nullptr;
  void* tflux = nullptr;
  void* tvc = nullptr;
  void* tfv = nullptr;
  double* tv = nullptr;   // [10N] direction and product staging
  // reverse-mode residual derivative workspace (allocated on first use):
  // adjoints of the reconstructed face states [16][F], of the cell fields
  // [NQ][N] and unlimited gradients [3 NQ][N], and the limiter bounds'
  // source cells and adjoints [2 NQ][N]
  double* aF = nullptr;
  double* aS = nullptr;   // [16][F] adjoints of the TVD gradient projections
  double* aQ = nullptr;
  double* aG = nullptr;
  int* aSrc = nullptr;
  double* aVal = nullptr;
  unsigned char* hbZoneBuf = nullptr;  // owner of m.hbZone
  // launch choices, set by the autotuner (ics_autotune) or left at the
  // defaults that the hand sweeps picked
  int tuneFaceBs = 128, tuneGradBs = 128, tuneMgsBlocks = 608, tuneFused = 1, tuneRevRows = 1;
  // exact Jacobian of the residual source: stencil CSR (two face hops plus
  // Harmonic Balance partners), transpose positions, colouring, blocks
  int* xptr = nullptr;
  int* xcol = nullptr;
  int* xtpos = nullptr;
  int* xcolour = nullptr;
  double* xblk = nullptr;  // [nnz][25]
  long long xnnz = 0;
  int xncol = 0;
  bool haveExact = false;
  // passive scalar transport: s, rhoS (+ old levels) [N], boundary s [B],
  // per-patch BC (fixed flag, value), face terms and the 1x1-block matrix
  bool scalarOn = false;
  double Ds = 0;
  int reconS = 0;
  double* ss = nullptr;
  double* ssB = nullptr;
  double* srhoS = nullptr;
  double* srhoS0 = nullptr;
  double* srhoS00 = nullptr;
  double* sgrad = nullptr;    // [3][N] reconstruction gradient of s
  double* sgradL = nullptr;   // [3][N] Gauss gradient of s (laplacian correction)
  double* sface = nullptr;    // [5][F+B]: flux - laplacian, upper, lower, owner diag, neighbour diag
  double* sblk = nullptr;     // [nslots*32]
  double* sdg = nullptr;      // [N]
  double* srD = nullptr;      // [N]
  double* ssrc = nullptr;     // [N]
  int* sFixed = nullptr;      // [npatches]
  double* sValue = nullptr;   // [npatches]
  // scratch
  double* scratch = nullptr;  // generic [N*5] doubles
  int* ibuf = nullptr;        // [N] flags
  // measurement
  long long launches = 0;
  bool prof = false;
  std::vector<cudaEvent_t> evPool;
  size_t evUsed = 0;
  std::vector<int> evKind;  // kind of each recorded pair
  double profMs[ICS_K_COUNT] = {};
  long long profN[ICS_K_COUNT] = {};
  cudaEvent_t tStart = nullptr, tStop = nullptr;
  // one GMRES restart cycle captured as a CUDA graph (key = precision*1000 + m)
  cudaGraphExec_t cycleExec = nullptr;
  int cycleKey = -1;
  long long cycleLaunches = 0;
  // independent cases stacked in this handle (ics_set_cases); n == 0: off
  CaseSet cases;
};

inline void drop_graphs(Handle& h) {
  if (h.cycleExec) cudaGraphExecDestroy(h.cycleExec);
  h.cycleExec = nullptr;
  h.cycleKey = -1;
}

// Times one kernel launch of class `kind` when profiling is on; counts it always.
struct Launch {
  Handle& h;
  int kind;
  cudaEvent_t stop = nullptr;
  Launch(Handle& hh, int k);
  ~Launch();
};

// ------------------------------------------------------------------ kernels
void launch_fields(Handle& h);
void launch_grad(Handle& h);
void launch_face_flux(Handle& h);
void launch_residual(Handle& h, double serRatio, bool applySer);
void launch_jacobian(Handle& h);
// the off-diagonal slots expanded to 25 FP64 entries, [nslots][25][32]
void launch_expand_slots(Handle& h, double* out);
void launch_update(Handle& h, int* boundedDev);
void launch_bc(Handle& h);
void launch_mrf_bc(Handle& h);
void launch_set_primitive(Handle& h);
void launch_derive_primitive(Handle& h);
void launch_bound_local_timestep(Handle& h);
void launch_viscous(Handle& h);
// Jacobian-vector product of the residual source: out = d(R V)/dW v at the
// current state with the boundary values held fixed (v, out device [N][5])
void launch_residual_tangent(Handle& h, const double* v, double* out);
// its transpose by reverse mode (out = (d(R V)/dW)^T u, device [N][5]),
// recomputing the fields and limited gradients; the empty string when the
// configuration is covered, else why not
void launch_residual_vjp(Handle& h, const double* u, double* out);
std::string residual_vjp_unsupported(const Handle& h);
// matrix-free Krylov solves (device FP64 [N][5] right-hand side and solution)
// and the patch pressure force with its gradient (device [N][5] or nullptr)
int adjoint_solve(Handle& h, const double* g, double* psi, const ics_krylov_opts& o, ics_krylov_result* res);
int tangent_solve(Handle& h, const double* b, double* x, const ics_krylov_opts& o, ics_krylov_result* res);
double pressure_force(Handle& h, int patch, const double dir[3], double* dJdW_dev);
// passive scalar: face terms + matrix rows at the current flow state, the
// scalar GMRES solve (increment in dx, device [N]) and the state update
void launch_scalar_assembly(Handle& h);
int scalar_gmres(Handle& h, double* dx, ics_solver_perf* perf);
void launch_scalar_update(Handle& h, const double* dx);
void launch_scalar_bc(Handle& h);
// exact Jacobian by coloured tangents; products with it and its transpose
void build_exact_pattern(Handle& h);
void free_exact(Handle& h);
void assemble_exact(Handle& h);
void exact_vjp(Handle& h, const double* u, double* y);
void exact_jvp(Handle& h, const double* x, double* y);

// independent cases stacked in one handle (k_cases.cu): set up the per-case
// reductions and state, release them, one GMRES solve of every active case
// (caseStatus [n]: ICS_OK, ICS_ERR_BREAKDOWN or ICS_ERR_NONFINITE per case;
// the return value reports a sweep that gave up), the per-case rho L2 sums
// of the last residual (host mirror) and the SER factors' upload
void set_cases(Handle& h, int n, const int* start);
void free_cases(Handle& h);
int gmres_cases(Handle& h, std::vector<int>& caseStatus);
void case_l2(Handle& h);
void case_upload_ser(Handle& h);

// linear algebra: precision-dispatched (mixed = FP32 blocks and vectors)
void spmv(Handle& h, const void* x, void* y);
int precondition(Handle& h, void* r);
// fills *perf (maximum over instances) and initRes (per instance, [5*J + k])
int gmres_solve(Handle& h, ics_solver_perf* perf, std::vector<double>& initRes);
// the autotuner's measurements on the handle's assembled system (ms per
// candidate) for the Krylov side and the residual side; they set the tune*
// fields to the fastest candidates
void autotune_linalg(Handle& h, std::vector<std::pair<std::string, double>>& log);
void autotune_residual(Handle& h, std::vector<std::pair<std::string, double>>& log);
// fields with a reconstruction gradient (bit k = q field k) and the MUSCL limiter kind
unsigned grad_mask(const Handle& h, int* limited);
void to_vec(Handle& h, const double* src, void* dst);   // FP64 -> Krylov type
void sweep_probe(Handle& h, const int* order, int count, int spin_limit);
void from_vec(Handle& h, const void* src, double* dst); // Krylov type -> FP64

inline int prec(const Handle& h) { return h.cfg.c.precision; }
// w = M^-1 A (x / beta) with v = x / beta stored in vout, by the fused LU-SGS
// operator passes; false (nothing launched) where they do not apply
bool fused_operator(Handle& h, const void* x, void* w, void* vout);
// element stride between consecutive Krylov basis vectors (5N rounded up to 64)
inline size_t kstride(const Handle& h) { return ((5ull * h.m.N + 63) / 64) * 64; }
inline size_t vbytes(const Handle& h) { return prec(h) == ICS_PREC_MIXED ? 4 : 8; }

#define ICS_CUDA(call)                                                    \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) throw ::ics::CudaError(e_, #call, __FILE__, __LINE__); \
  } while (0)

struct CudaError {
  cudaError_t e;
  const char* what;
  const char* file;
  int line;
  CudaError(cudaError_t e_, const char* w, const char* f, int l) : e(e_), what(w), file(f), line(l) {}
};

// launch a kernel as class `kind` (timed when profiling is on)
#define ICS_LAUNCH(hnd, kind, ...)    \
  do {                                \
    ::ics::Launch ics_l_((hnd), kind); \
    __VA_ARGS__;                      \
  } while (0)

inline int grid_for(long n, int bs) {
  long g = (n + bs - 1) / bs;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace ics
