// Stand-in for ICSFoam's coupledMatrix and its solver base class
// (src/coupledMatrix/coupledMatrix.H, coupledMatrixSolver.C): the selection
// table keyed by "solver", the solver constructor arguments and the
// delta-form solveDelta virtual with its residualsIO result.
#pragma once
#include "openfoam_stub.H"

namespace Foam {

struct residualsIO {
  List<scalar> initRes, finalRes;
  label nIterations = 0;
  bool converged = false;
};

class coupledMatrix {
  const fvMesh& mesh_;
  label nScal_, nVect_;

 public:
  coupledMatrix(const fvMesh& mesh, label nScal, label nVect) : mesh_(mesh), nScal_(nScal), nVect_(nVect) {}
  const fvMesh& mesh() const { return mesh_; }
  label nScal() const { return nScal_; }
  label nVect() const { return nVect_; }

  class solver {
   protected:
    const coupledMatrix& matrix_;
    dictionary controlDict_;

   public:
    declareRunTimeSelectionTable(autoPtr, solver, dictionary, (const dictionary& dict, const coupledMatrix& matrix),
                                 (dict, matrix));
    solver(const word&, const dictionary& dict, const coupledMatrix& matrix) : matrix_(matrix), controlDict_(dict) {}
    virtual ~solver() = default;
    static autoPtr<solver> New(const dictionary& dict, const coupledMatrix& matrix) {
      const word name = dict.get<word>("solver");
      auto it = dictionaryConstructorTable().find(name);
      if (it == dictionaryConstructorTable().end())
        FatalErrorInFunction << "Unknown solver type " << name << exit(FatalError);
      return it->second(dict.subDict(name), matrix);
    }
    const coupledMatrix& matrix() const { return matrix_; }
    virtual residualsIO solveDelta(PtrList<volScalarField>& sW, PtrList<volVectorField>& vW,
                                   const PtrList<scalarField>& sSource, const PtrList<vectorField>& vSource,
                                   PtrList<volScalarField>& dsW, PtrList<volVectorField>& dvW) const = 0;
  };
};

}  // namespace Foam
