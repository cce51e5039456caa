// OpenFOAM-side shim of the GB300 path: runtime-selectable convective flux
// schemes (AUSMPlusUpGPU, HLLCGPU, ROEGPU) and a coupled-matrix solver
// (GMRESGPU) that forward to the C ABI of include/icsfoam_gb300.h, so that an
// ICSFoam case switches to the GPU by name in its dictionaries:
//
//   fvSchemes  convectiveFluxScheme { fluxScheme HLLCGPU; }
//   fvSolution flowSolver { solver GMRESGPU; GMRESGPU { preconditioner LUSGS;
//                           nDirections 8; maxIter 5; tolerance 1e-12; relTol 1e-2; } }
//
// The flux schemes register in convectiveFluxScheme's selection table
// (convectiveFluxScheme.H:117-130, as ausmPlusUpFluxScheme.C:41-42 does) and
// the solver in coupledMatrix::solver's (coupledMatrix.H:94-214,
// coupledMatrixSolver.C:41-67).  One GPU case (ics_handle) per mesh is shared
// by the mesh's flux scheme and solver: the flux scheme uploads the mesh once,
// pushes the current conservative state and boundary values before each
// flux evaluation, and the solver solves the GPU case's own system at that
// state (residual source, Jacobian and GMRES on the device; the host-side
// blocks are not used) and hands back the increment in the reference's
// unknown order (rho, rhoE scalars, then rhoU).
//
// Built with wmake inside ICSFoam against OpenFOAM v2112 (Make/files,
// Make/options); the repository's tests compile and run it against minimal
// stand-ins of the OpenFOAM types.
#pragma once

#include <memory>
#include <vector>

#include "convectiveFluxScheme.H"
#include "coupledMatrix.H"
#include "icsfoam_gb300.h"

namespace Foam {
namespace gb300 {

// FatalError with the handle's message when a C-ABI call fails
void check(ics_handle h, int status, const char* what);

// The patch kind and values the GPU path applies to patch i: from the p, U
// and T boundary-condition types of the case (the one place that maps
// OpenFOAM BC names to ICS_PATCH_* kinds).
ics_patch_desc patchDescription(const psiThermo& thermo, label patchi);

// One GPU case per mesh
class Case {
 public:
  static Case& of(const fvMesh& mesh, const psiThermo& thermo, const ics_config& cfg);
  static Case* find(const fvMesh& mesh);
  ~Case();
  ics_handle handle() const { return h_; }
  // conservative state and boundary values of the current fields
  void pushState(const volScalarField& rho, const volVectorField& U, const volScalarField& p,
                 const volScalarField& T);
  label nFaces() const { return nFaces_; }
  label nBFaces() const { return nBFaces_; }
  // the non-empty patches in the order the C ABI lists their faces
  const std::vector<label>& patches() const { return patches_; }
  // the linear-solver entries of the handle's configuration (GMRESGPU)
  void setSolver(int preconditioner, int nDirections, int maxIter, double tolerance, double relTol,
                 int precision);

 private:
  Case(const fvMesh& mesh, const psiThermo& thermo, const ics_config& cfg);
  const fvMesh& mesh_;
  ics_handle h_ = nullptr;
  double Cv_ = 0.0;  // Cp - R of the handle's thermo
  ics_config cfg_;   // the handle's current configuration
  label nFaces_ = 0, nBFaces_ = 0;
  std::vector<label> patches_;
};

// ics_config from the dictionaries a case gives the flux scheme: thermo
// constants, reconstruct(...) schemes and the GPU scheme's flux choice
ics_config configFor(const psiThermo& thermo, const dictionary& fluxDict, int fluxScheme);

template <int FLUX>
class GPUFluxScheme : public convectiveFluxScheme {
 public:
  GPUFluxScheme(const word& type, const dictionary& dict, const psiThermo& thermo, const volScalarField& rho,
                const volVectorField& U, const volScalarField& p);
  void calcFlux(surfaceScalarField& phi, surfaceVectorField& phiUp, surfaceScalarField& phiEp) override;

 private:
  Case& case_;
};

class AUSMPlusUpGPU : public GPUFluxScheme<ICS_FLUX_AUSMPLUSUP> {
 public:
  TypeName("AUSMPlusUpGPU");
  AUSMPlusUpGPU(const dictionary& dict, const psiThermo& thermo, const volScalarField& rho, const volVectorField& U,
                const volScalarField& p)
      : GPUFluxScheme(typeName_(), dict, thermo, rho, U, p) {}
};
class HLLCGPU : public GPUFluxScheme<ICS_FLUX_HLLC> {
 public:
  TypeName("HLLCGPU");
  HLLCGPU(const dictionary& dict, const psiThermo& thermo, const volScalarField& rho, const volVectorField& U,
          const volScalarField& p)
      : GPUFluxScheme(typeName_(), dict, thermo, rho, U, p) {}
};
class ROEGPU : public GPUFluxScheme<ICS_FLUX_ROE> {
 public:
  TypeName("ROEGPU");
  ROEGPU(const dictionary& dict, const psiThermo& thermo, const volScalarField& rho, const volVectorField& U,
         const volScalarField& p)
      : GPUFluxScheme(typeName_(), dict, thermo, rho, U, p) {}
};

// coupledMatrix::solver whose solveDelta runs the GPU case's GMRES
class GMRESGPU : public coupledMatrix::solver {
 public:
  TypeName("GMRESGPU");
  GMRESGPU(const dictionary& dict, const coupledMatrix& matrix);
  residualsIO solveDelta(PtrList<volScalarField>& sW, PtrList<volVectorField>& vW,
                         const PtrList<scalarField>& sSource, const PtrList<vectorField>& vSource,
                         PtrList<volScalarField>& dsW, PtrList<volVectorField>& dvW) const override;

 private:
  int preconditioner_, nDirections_, maxIter_;
  double tolerance_, relTol_;
  int precision_;
};

}  // namespace gb300
}  // namespace Foam
