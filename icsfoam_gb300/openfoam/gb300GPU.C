// OpenFOAM-side shim of the GB300 path: see gb300GPU.H.
#include "gb300GPU.H"

#include <map>
#include <sstream>
#include <string>

namespace Foam {
namespace gb300 {

void check(ics_handle h, int status, const char* what) {
  if (status == ICS_OK) return;
  char msg[512] = "";
  if (h) ics_last_error(h, msg, sizeof(msg));
  FatalErrorInFunction << what << " failed with status " << status << ": " << msg << exit(FatalError);
}

// ----------------------------------------------------------------- Case
namespace {
std::map<const fvMesh*, std::unique_ptr<Case>>& registry() {
  static std::map<const fvMesh*, std::unique_ptr<Case>> r;
  return r;
}
void put(std::vector<double>& v, const vector& a) {
  v.push_back(a[0]);
  v.push_back(a[1]);
  v.push_back(a[2]);
}
}  // namespace

Case* Case::find(const fvMesh& mesh) {
  auto it = registry().find(&mesh);
  return it == registry().end() ? nullptr : it->second.get();
}

Case& Case::of(const fvMesh& mesh, const psiThermo& thermo, const ics_config& cfg) {
  if (Case* c = find(mesh)) {
    // a new flux scheme on a mesh that has a case: its entries, the solver's kept
    ics_config n = cfg;
    const ics_config& o = c->cfg_;
    n.solver = o.solver;
    n.preconditioner = o.preconditioner;
    n.n_directions = o.n_directions;
    n.max_iter = o.max_iter;
    n.min_iter = o.min_iter;
    n.tolerance = o.tolerance;
    n.rel_tol = o.rel_tol;
    n.precision = o.precision;
    check(c->h_, ics_set_config(c->h_, &n), "ics_set_config");
    c->cfg_ = n;
    return *c;
  }
  registry()[&mesh].reset(new Case(mesh, thermo, cfg));
  return *registry()[&mesh];
}

Case::Case(const fvMesh& mesh, const psiThermo& thermo, const ics_config& cfg)
    : mesh_(mesh), Cv_(cfg.Cp - cfg.R), cfg_(cfg) {
  const label N = mesh.nCells(), F = mesh.nInternalFaces();
  std::vector<double> Sf, Cf, C, bSf, bCf, bdc;
  std::vector<int32_t> bCell, bPatch;
  for (label f = 0; f < F; ++f) {
    put(Sf, mesh.Sf()[f]);
    put(Cf, mesh.Cf()[f]);
  }
  for (label c = 0; c < N; ++c) put(C, mesh.C()[c]);
  std::vector<ics_patch_desc> descs;
  const auto& bnd = mesh.boundary();
  for (label i = 0; i < (label)bnd.size(); ++i) {
    if (bnd[i].type == "empty") continue;
    const int32_t k = (int32_t)descs.size();
    descs.push_back(patchDescription(thermo, i));
    patches_.push_back(i);
    for (label j = 0; j < bnd[i].size(); ++j) {
      bCell.push_back(bnd[i].faceCells[j]);
      bPatch.push_back(k);
      put(bSf, bnd[i].Sf[j]);
      put(bCf, bnd[i].Cf[j]);
      bdc.push_back(bnd[i].deltaCoeffs[j]);
    }
  }
  nFaces_ = F;
  nBFaces_ = (label)bCell.size();
  ics_mesh_desc m = {};
  m.n_cells = N;
  m.n_faces = F;
  m.n_bfaces = nBFaces_;
  m.n_patches = (int32_t)descs.size();
  m.owner = mesh.owner().data();
  m.neighbour = mesh.neighbour().data();
  m.Sf = Sf.data();
  m.Cf = Cf.data();
  m.weights = mesh.weights().data();
  m.delta_coeffs = mesh.deltaCoeffs().data();
  m.nonorth_delta_coeffs = mesh.nonOrthDeltaCoeffs().data();
  m.C = C.data();
  m.V = mesh.V().data();
  m.b_cell = bCell.data();
  m.b_patch = bPatch.data();
  m.b_Sf = bSf.data();
  m.b_Cf = bCf.data();
  m.b_delta_coeffs = bdc.data();
  m.patches = descs.data();
  for (int d = 0; d < 3; ++d) m.solution_d[d] = mesh.solutionD()[d];
  check(nullptr, ics_create(&m, &cfg, &h_), "ics_create");
}

void Case::setSolver(int preconditioner, int nDirections, int maxIter, double tolerance, double relTol,
                     int precision) {
  ics_config n = cfg_;
  n.solver = ICS_SOLVER_GMRES;
  n.preconditioner = preconditioner;
  n.n_directions = nDirections;
  n.max_iter = maxIter;
  n.tolerance = tolerance;
  n.rel_tol = relTol;
  n.precision = precision;
  check(h_, ics_set_config(h_, &n), "ics_set_config");
  cfg_ = n;
}

Case::~Case() {
  if (h_) ics_destroy(h_);
}

void Case::pushState(const volScalarField& rho, const volVectorField& U, const volScalarField& p,
                     const volScalarField& T) {
  const label N = mesh_.nCells();
  std::vector<double> W(5 * (size_t)N);
  for (label c = 0; c < N; ++c) {
    const double r = rho.primitiveField()[c];
    const vector& u = U.primitiveField()[c];
    W[5 * c] = r;
    for (int k = 0; k < 3; ++k) W[5 * c + 1 + k] = r * u[k];
    // rhoE = rho (e + |U|^2 / 2), e = Cv T (sensibleInternalEnergy, Tref = 0)
    W[5 * c + 4] = r * (Cv_ * T.primitiveField()[c] + 0.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
  }
  std::vector<double> pb, Ub, Tb, phib;
  for (label i : patches_) {
    const auto& pa = mesh_.boundary()[i];
    for (label j = 0; j < pa.size(); ++j) {
      const vector& ub = U.boundaryField()[i][j];
      const double rb = rho.boundaryField()[i][j];
      pb.push_back(p.boundaryField()[i][j]);
      Tb.push_back(T.boundaryField()[i][j]);
      for (int k = 0; k < 3; ++k) Ub.push_back(ub[k]);
      phib.push_back(rb * (ub[0] * pa.Sf[j][0] + ub[1] * pa.Sf[j][1] + ub[2] * pa.Sf[j][2]));
    }
  }
  check(h_, ics_set_conservative(h_, W.data(), 0), "ics_set_conservative");
  check(h_, ics_set_boundary_state(h_, pb.data(), Ub.data(), Tb.data(), phib.data()), "ics_set_boundary_state");
}

// ------------------------------------------------------------ configuration
namespace {
// interpolationSchemes reconstruct(...) entry (with its gradSchemes entry)
int reconstruction(const dictionary& interp, const dictionary& grads, const word& field) {
  const word key = "reconstruct(" + field + ")";
  if (!interp.found(key)) return ICS_RECON_UPWIND;
  auto&& is = interp.lookup(key);
  word kind, gradName;
  is >> kind >> gradName;
  if (kind == "upwind") return ICS_RECON_UPWIND;
  if (kind == "vanLeer") return ICS_RECON_VANLEER;
  if (kind == "Minmod" || kind == "minmod") return ICS_RECON_MINMOD;
  if (kind == "linearUpwind") {
    const word gkey = grads.found(gradName) ? gradName : word("default");
    word g;
    if (grads.found(gkey)) {
      auto&& gs = grads.lookup(gkey);
      gs >> g;
    }
    if (g == "cellLimited<Venkatakrishnan>") return ICS_RECON_MUSCL_VENKATAKRISHNAN;
    if (g == "cellLimited" || g == "cellLimited<minmod>") return ICS_RECON_MUSCL_MINMOD;
  }
  FatalErrorInFunction << "Unsupported reconstruction " << kind << " for " << field << exit(FatalError);
  return ICS_RECON_UPWIND;
}
}  // namespace

ics_config configFor(const psiThermo& thermo, const dictionary& fluxDict, int fluxScheme) {
  ics_config c;
  ics_default_config(&c);
  c.R = thermo.R();
  c.Cp = thermo.Cp();
  c.flux_scheme = fluxScheme;
  c.low_mach_ausm = fluxDict.getOrDefault<int>("lowMachAusm", 1);
  c.entropy_fix_coeff = fluxDict.getOrDefault<double>("entropyFixCoeff", 0.05);
  if (fluxDict.found("interpolationSchemes")) {
    const dictionary& interp = fluxDict.subDict("interpolationSchemes");
    const dictionary empty;
    const dictionary& grads = fluxDict.found("gradSchemes") ? fluxDict.subDict("gradSchemes") : empty;
    c.recon_rho = reconstruction(interp, grads, "rho");
    c.recon_U = reconstruction(interp, grads, "U");
    c.recon_T = reconstruction(interp, grads, "T");
  }
  return c;
}

// ------------------------------------------------------------ flux schemes
template <int FLUX>
GPUFluxScheme<FLUX>::GPUFluxScheme(const word& type, const dictionary& dict, const psiThermo& thermo,
                                   const volScalarField& rho, const volVectorField& U, const volScalarField& p)
    : convectiveFluxScheme(type, dict, thermo, rho, U, p),
      case_(Case::of(rho.mesh(), thermo, configFor(thermo, dict, FLUX))) {}

template <int FLUX>
void GPUFluxScheme<FLUX>::calcFlux(surfaceScalarField& phi, surfaceVectorField& phiUp, surfaceScalarField& phiEp) {
  case_.pushState(rho(), U(), p(), thermo().T());
  const label F = case_.nFaces(), B = case_.nBFaces();
  std::vector<double> f(F + B), fu(3 * (size_t)(F + B)), fe(F + B);
  check(case_.handle(), ics_calc_flux(case_.handle(), f.data(), fu.data(), fe.data()), "ics_calc_flux");
  for (label i = 0; i < F; ++i) {
    phi.primitiveFieldRef()[i] = f[i];
    phiUp.primitiveFieldRef()[i] = vector(fu[3 * i], fu[3 * i + 1], fu[3 * i + 2]);
    phiEp.primitiveFieldRef()[i] = fe[i];
  }
  label b = F;
  for (label pi : case_.patches()) {
    for (label j = 0; j < mesh().boundary()[pi].size(); ++j, ++b) {
      phi.boundaryFieldRef()[pi][j] = f[b];
      phiUp.boundaryFieldRef()[pi][j] = vector(fu[3 * b], fu[3 * b + 1], fu[3 * b + 2]);
      phiEp.boundaryFieldRef()[pi][j] = fe[b];
    }
  }
}

template class GPUFluxScheme<ICS_FLUX_AUSMPLUSUP>;
template class GPUFluxScheme<ICS_FLUX_HLLC>;
template class GPUFluxScheme<ICS_FLUX_ROE>;

addToRunTimeSelectionTable(convectiveFluxScheme, AUSMPlusUpGPU, dictionary);
addToRunTimeSelectionTable(convectiveFluxScheme, HLLCGPU, dictionary);
addToRunTimeSelectionTable(convectiveFluxScheme, ROEGPU, dictionary);

// ------------------------------------------------------------------ solver
GMRESGPU::GMRESGPU(const dictionary& dict, const coupledMatrix& matrix)
    : coupledMatrix::solver(typeName_(), dict, matrix) {
  const std::string pc = dict.getOrDefault<std::string>("preconditioner", "LUSGS");
  preconditioner_ = pc == "LUSGS" ? ICS_PC_LUSGS : (pc == "Jacobi" ? ICS_PC_JACOBI : ICS_PC_NONE);
  if (pc != "LUSGS" && pc != "Jacobi" && pc != "none")
    FatalErrorInFunction << "Unknown preconditioner " << pc << exit(FatalError);
  nDirections_ = dict.get<int>("nDirections");
  maxIter_ = dict.getOrDefault<int>("maxIter", 1000);
  tolerance_ = dict.get<double>("tolerance");
  relTol_ = dict.get<double>("relTol");
  const std::string prec = dict.getOrDefault<std::string>("precision", "fp64");
  precision_ = prec == "mixed" ? ICS_PREC_MIXED : ICS_PREC_FP64;
}

residualsIO GMRESGPU::solveDelta(PtrList<volScalarField>&, PtrList<volVectorField>&, const PtrList<scalarField>&,
                                 const PtrList<vectorField>&, PtrList<volScalarField>& dsW,
                                 PtrList<volVectorField>& dvW) const {
  Case* c = Case::find(matrix().mesh());
  if (!c)
    FatalErrorInFunction << "GMRESGPU needs a GPU convective flux scheme on the same mesh" << exit(FatalError);
  ics_handle h = c->handle();
  // the handle keeps the flux scheme's entries; the solver's replace its own
  c->setSolver(preconditioner_, nDirections_, maxIter_, tolerance_, relTol_, precision_);
  const label N = matrix().mesh().nCells();
  std::vector<double> dW(5 * (size_t)N);
  check(h, ics_residual(h, nullptr), "ics_residual");
  check(h, ics_assemble_jacobian(h), "ics_assemble_jacobian");
  ics_solver_perf perf;
  const int st = ics_solve_increment(h, &perf, dW.data());
  if (st != ICS_OK && st != ICS_ERR_BREAKDOWN) check(h, st, "ics_solve_increment");
  // the reference's unknowns: scalars rho, rhoE, then the vector rhoU
  for (label k = 0; k < N; ++k) {
    dsW[0]->primitiveFieldRef()[k] = dW[5 * k];
    dsW[1]->primitiveFieldRef()[k] = dW[5 * k + 4];
    dvW[0]->primitiveFieldRef()[k] = vector(dW[5 * k + 1], dW[5 * k + 2], dW[5 * k + 3]);
  }
  residualsIO r;
  r.initRes.assign(perf.init_res, perf.init_res + 5);
  r.finalRes.assign(perf.final_res, perf.final_res + 5);
  r.nIterations = perf.n_iterations;
  r.converged = perf.converged != 0;
  return r;
}

addToRunTimeSelectionTable(coupledMatrix::solver, GMRESGPU, dictionary);

}  // namespace gb300
}  // namespace Foam
