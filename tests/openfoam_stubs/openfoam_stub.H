// Minimal stand-ins for the OpenFOAM v2112 and ICSFoam types the GPU shim
// (icsfoam_gb300/openfoam) uses, so that the shim compiles and runs in a test
// without OpenFOAM.  Only the members the shim touches exist; their meaning
// follows the real classes (fvMesh addressing and geometry, geometric fields
// with per-patch boundary fields, dictionaries, runtime-selection tables).
#pragma once

#include <array>
#include <cmath>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace Foam {

using word = std::string;
using label = int;
using scalar = double;

struct vector {
  double v[3] = {0, 0, 0};
  vector() = default;
  vector(double a, double b, double c) : v{a, b, c} {}
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
  double x() const { return v[0]; }
  double y() const { return v[1]; }
  double z() const { return v[2]; }
};

template <class T>
using Field = std::vector<T>;
using scalarField = Field<scalar>;
using vectorField = Field<vector>;
using labelUList = std::vector<label>;
template <class T>
using List = std::vector<T>;
template <class T>
using autoPtr = std::unique_ptr<T>;
template <class T>
using PtrList = std::vector<std::unique_ptr<T>>;

// FatalError ... exit(FatalError): a thrown error in the stand-in
struct FatalErrorType {
  std::ostringstream msg;
};
struct FatalExit {};
inline FatalExit exit(FatalErrorType&) { return {}; }
struct FatalErrorStream {
  std::ostringstream os;
  template <class T>
  FatalErrorStream& operator<<(const T& v) {
    os << v;
    return *this;
  }
  FatalErrorStream& operator<<(FatalExit) { throw std::runtime_error(os.str()); }
};
extern FatalErrorType FatalError;
#define FatalErrorInFunction (::Foam::FatalErrorStream())

// dictionary: entries as strings, sub-dictionaries by name
class dictionary {
 public:
  std::map<word, std::string> entries;
  std::map<word, dictionary> dicts;
  bool found(const word& k) const { return entries.count(k) || dicts.count(k); }
  const dictionary& subDict(const word& k) const {
    auto it = dicts.find(k);
    if (it == dicts.end()) throw std::runtime_error("keyword " + k + " is undefined");
    return it->second;
  }
  template <class T>
  T get(const word& k) const {
    auto it = entries.find(k);
    if (it == entries.end()) throw std::runtime_error("keyword " + k + " is undefined");
    std::istringstream is(it->second);
    T v{};
    is >> v;
    return v;
  }
  // the entry as a token stream (OpenFOAM: ITstream& lookup(const word&))
  std::istringstream lookup(const word& k) const {
    auto it = entries.find(k);
    if (it == entries.end()) throw std::runtime_error("keyword " + k + " is undefined");
    return std::istringstream(it->second);
  }
  template <class T>
  T getOrDefault(const word& k, const T& d) const {
    return entries.count(k) ? get<T>(k) : d;
  }
};

// boundary patches of the mesh
struct fvPatch {
  word name, type;  // type: "patch", "wall", "empty", ...
  labelUList faceCells;
  vectorField Sf, Cf;
  scalarField deltaCoeffs;
  label size() const { return (label)faceCells.size(); }
};

class fvMesh {
 public:
  label nCells_ = 0;
  labelUList owner_, neighbour_;
  vectorField Sf_, Cf_, C_;
  scalarField V_, weights_, deltaCoeffs_, nonOrthDeltaCoeffs_;
  std::vector<fvPatch> boundary_;
  std::array<label, 3> solutionD_{{1, 1, 1}};
  label nCells() const { return nCells_; }
  label nInternalFaces() const { return (label)owner_.size(); }
  const labelUList& owner() const { return owner_; }
  const labelUList& neighbour() const { return neighbour_; }
  const vectorField& Sf() const { return Sf_; }
  const vectorField& Cf() const { return Cf_; }
  const vectorField& C() const { return C_; }
  const scalarField& V() const { return V_; }
  const scalarField& weights() const { return weights_; }
  const scalarField& deltaCoeffs() const { return deltaCoeffs_; }
  const scalarField& nonOrthDeltaCoeffs() const { return nonOrthDeltaCoeffs_; }
  const std::vector<fvPatch>& boundary() const { return boundary_; }
  const std::array<label, 3>& solutionD() const { return solutionD_; }
};

// geometric fields: internal values and one value list per patch
template <class T>
class GeometricField {
 public:
  const fvMesh* mesh_ = nullptr;
  word name_;
  Field<T> internal;
  std::vector<Field<T>> boundary;
  GeometricField(const word& n, const fvMesh& m, label size) : mesh_(&m), name_(n), internal(size) {
    for (const auto& p : m.boundary()) boundary.emplace_back(p.size());
  }
  const fvMesh& mesh() const { return *mesh_; }
  const word& name() const { return name_; }
  Field<T>& primitiveFieldRef() { return internal; }
  const Field<T>& primitiveField() const { return internal; }
  std::vector<Field<T>>& boundaryFieldRef() { return boundary; }
  const std::vector<Field<T>>& boundaryField() const { return boundary; }
};
using volScalarField = GeometricField<scalar>;
using volVectorField = GeometricField<vector>;
using surfaceScalarField = GeometricField<scalar>;
using surfaceVectorField = GeometricField<vector>;

// perfectGas + hConst thermo with the boundary conditions of p, U and T
class psiThermo {
 public:
  const fvMesh& mesh_;
  scalar R_, Cp_;
  volScalarField T_;
  // per patch: the BC of the case in the shim's vocabulary (patch kind and values)
  struct PatchBC {
    int kind = 1;
    double p = 0, T = 0, U[3] = {0, 0, 0}, p0 = 0, T0 = 0;
  };
  std::vector<PatchBC> bcs;
  psiThermo(const fvMesh& m, scalar R, scalar Cp) : mesh_(m), R_(R), Cp_(Cp), T_("T", m, m.nCells()) {}
  const volScalarField& T() const { return T_; }
  volScalarField& T() { return T_; }
  scalar R() const { return R_; }
  scalar Cp() const { return Cp_; }
};

}  // namespace Foam

// ---- runtime selection (the pattern of OpenFOAM's runTimeSelectionTables.H)
#define TypeName(N)                            \
  static const char* typeName_() { return N; } \
  virtual const Foam::word type() const { return N; }

#define declareRunTimeSelectionTable(ptr, base, tab, args, pars)                 \
  using tab##ConstructorPtr = ptr<base> (*) args;                               \
  static std::map<Foam::word, tab##ConstructorPtr>& tab##ConstructorTable() {   \
    static std::map<Foam::word, tab##ConstructorPtr> t;                         \
    return t;                                                                   \
  }                                                                             \
  template <class Derived>                                                      \
  struct add##tab##ConstructorToTable {                                         \
    static ptr<base> New args { return ptr<base>(new Derived pars); }           \
    explicit add##tab##ConstructorToTable(const Foam::word& n) {                \
      tab##ConstructorTable()[n] = New;                                         \
    }                                                                           \
  };

#define ICS_CAT2(a, b) a##b
#define ICS_CAT(a, b) ICS_CAT2(a, b)
#define addToRunTimeSelectionTable(base, derived, tab)                                      \
  static base::add##tab##ConstructorToTable<derived> ICS_CAT(add_##derived##_, __LINE__)( \
      derived::typeName_())
