// Stand-in for ICSFoam's convectiveFluxScheme base class
// (src/convectiveFluxSchemes/convectiveFluxScheme/convectiveFluxScheme.H):
// the same constructor arguments, selection table and calcFlux virtual.
#pragma once
#include "openfoam_stub.H"

namespace Foam {

class convectiveFluxScheme {
  const dictionary& dict_;
  const fvMesh& mesh_;
  const psiThermo& thermo_;
  const volScalarField& rho_;
  const volVectorField& U_;
  const volScalarField& p_;

 public:
  TypeName("convectiveFluxScheme");
  declareRunTimeSelectionTable(autoPtr, convectiveFluxScheme, dictionary,
                               (const dictionary& dict, const psiThermo& thermo, const volScalarField& rho,
                                const volVectorField& U, const volScalarField& p),
                               (dict, thermo, rho, U, p));
  convectiveFluxScheme(const word&, const dictionary& dict, const psiThermo& thermo, const volScalarField& rho,
                       const volVectorField& U, const volScalarField& p)
      : dict_(dict), mesh_(rho.mesh()), thermo_(thermo), rho_(rho), U_(U), p_(p) {}
  virtual ~convectiveFluxScheme() = default;
  // selection by fvSchemes/convectiveFluxScheme/fluxScheme
  static autoPtr<convectiveFluxScheme> New(const dictionary& dict, const psiThermo& thermo,
                                           const volScalarField& rho, const volVectorField& U,
                                           const volScalarField& p) {
    const word name = dict.get<word>("fluxScheme");
    auto it = dictionaryConstructorTable().find(name);
    if (it == dictionaryConstructorTable().end())
      FatalErrorInFunction << "Unknown convectiveFluxScheme type " << name << exit(FatalError);
    return it->second(dict, thermo, rho, U, p);
  }
  const dictionary& dict() const { return dict_; }
  const fvMesh& mesh() const { return mesh_; }
  const psiThermo& thermo() const { return thermo_; }
  const volScalarField& rho() const { return rho_; }
  const volVectorField& U() const { return U_; }
  const volScalarField& p() const { return p_; }
  virtual void calcFlux(surfaceScalarField& phi, surfaceVectorField& phiUp, surfaceScalarField& phiEp) = 0;
};

}  // namespace Foam
