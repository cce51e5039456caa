// Runs the OpenFOAM-side GPU shim (icsfoam_gb300/openfoam/gb300GPU.C) the
// way dbnsFoam would, on the OpenFOAM stand-ins: reads a mesh and a state
// written by the test (binary, see tests/test_openfoam_shim.py), selects the
// flux scheme and the solver BY NAME through the runtime-selection tables,
// calls calcFlux and solveDelta, and writes the fluxes and the increment.
//
// usage: shim_driver case.bin out.bin fluxSchemeName solverName
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>

#include "gb300GPU.H"

namespace Foam {
FatalErrorType FatalError;
namespace gb300 {
// the stand-in thermo carries the case's boundary conditions as patch kinds
ics_patch_desc patchDescription(const psiThermo& thermo, label patchi) {
  const auto& b = thermo.bcs[patchi];
  ics_patch_desc d = {};
  d.kind = b.kind;
  d.is_wall = thermo.mesh_.boundary()[patchi].type == "wall";
  d.p = b.p;
  d.T = b.T;
  for (int k = 0; k < 3; ++k) d.U[k] = b.U[k];
  d.p0 = b.p0;
  d.T0 = b.T0;
  return d;
}
}  // namespace gb300
}  // namespace Foam

using namespace Foam;

namespace {
struct Reader {
  std::ifstream in;
  explicit Reader(const char* path) : in(path, std::ios::binary) {
    if (!in) throw std::runtime_error(std::string("cannot open ") + path);
  }
  template <class T>
  T one() {
    T v;
    in.read(reinterpret_cast<char*>(&v), sizeof(T));
    return v;
  }
  template <class T>
  std::vector<T> many(size_t n) {
    std::vector<T> v(n);
    in.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
    return v;
  }
  vectorField vecs(size_t n) {
    auto a = many<double>(3 * n);
    vectorField v(n);
    for (size_t i = 0; i < n; ++i) v[i] = vector(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
    return v;
  }
  std::string name() {
    auto c = many<char>(32);
    return std::string(c.data(), strnlen(c.data(), 32));
  }
};
}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s case.bin out.bin fluxScheme solver\n", argv[0]);
    return 2;
  }
  try {
    Reader r(argv[1]);
    fvMesh mesh;
    const int N = r.one<int32_t>(), F = r.one<int32_t>(), P = r.one<int32_t>();
    const double R = r.one<double>(), Cp = r.one<double>();
    mesh.nCells_ = N;
    {
      auto o = r.many<int32_t>(F), n = r.many<int32_t>(F);
      mesh.owner_.assign(o.begin(), o.end());
      mesh.neighbour_.assign(n.begin(), n.end());
    }
    mesh.Sf_ = r.vecs(F);
    mesh.Cf_ = r.vecs(F);
    mesh.weights_ = r.many<double>(F);
    mesh.deltaCoeffs_ = r.many<double>(F);
    mesh.nonOrthDeltaCoeffs_ = r.many<double>(F);
    mesh.C_ = r.vecs(N);
    mesh.V_ = r.many<double>(N);
    std::vector<psiThermo::PatchBC> bcs;
    for (int i = 0; i < P; ++i) {
      fvPatch pa;
      pa.name = r.name();
      pa.type = r.name();
      psiThermo::PatchBC bc;
      bc.kind = r.one<int32_t>();
      bc.p = r.one<double>();
      bc.T = r.one<double>();
      for (int k = 0; k < 3; ++k) bc.U[k] = r.one<double>();
      bc.p0 = r.one<double>();
      bc.T0 = r.one<double>();
      const int n = r.one<int32_t>();
      auto fc = r.many<int32_t>(n);
      pa.faceCells.assign(fc.begin(), fc.end());
      pa.Sf = r.vecs(n);
      pa.Cf = r.vecs(n);
      pa.deltaCoeffs = r.many<double>(n);
      mesh.boundary_.push_back(pa);
      bcs.push_back(bc);
    }
    psiThermo thermo(mesh, R, Cp);
    thermo.bcs = bcs;
    volScalarField rho("rho", mesh, N), p("p", mesh, N);
    volVectorField U("U", mesh, N);
    rho.internal = r.many<double>(N);
    U.internal = r.vecs(N);
    p.internal = r.many<double>(N);
    thermo.T().internal = r.many<double>(N);
    for (int i = 0; i < P; ++i) {
      const size_t n = mesh.boundary_[i].size();
      rho.boundary[i] = r.many<double>(n);
      U.boundary[i] = r.vecs(n);
      p.boundary[i] = r.many<double>(n);
      thermo.T().boundary[i] = r.many<double>(n);
    }
    // fvSchemes/convectiveFluxScheme (with the reconstruction entries the
    // GPU scheme reads) and fvSolution/flowSolver
    dictionary fluxDict;
    fluxDict.entries["fluxScheme"] = argv[3];
    dictionary interp, grads;
    for (const char* f : {"rho", "U", "T"}) interp.entries[std::string("reconstruct(") + f + ")"] = "linearUpwind grad";
    grads.entries["grad"] = "cellLimited<Venkatakrishnan> Gauss linear 1";
    fluxDict.dicts["interpolationSchemes"] = interp;
    fluxDict.dicts["gradSchemes"] = grads;
    auto scheme = convectiveFluxScheme::New(fluxDict, thermo, rho, U, p);
    surfaceScalarField phi("phi", mesh, F), phiE("phiE", mesh, F);
    surfaceVectorField phiU("phiUp", mesh, F);
    scheme->calcFlux(phi, phiU, phiE);

    dictionary solverDict, gm;
    solverDict.entries["solver"] = argv[4];
    gm.entries["preconditioner"] = "LUSGS";
    gm.entries["nDirections"] = "8";
    gm.entries["maxIter"] = "5";
    gm.entries["tolerance"] = "1e-12";
    gm.entries["relTol"] = "1e-2";
    solverDict.dicts[argv[4]] = gm;
    coupledMatrix eqSystem(mesh, 2, 1);
    auto solver = coupledMatrix::solver::New(solverDict, eqSystem);
    PtrList<volScalarField> sW, dsW;
    PtrList<volVectorField> vW, dvW;
    PtrList<scalarField> sSrc;
    PtrList<vectorField> vSrc;
    for (int k = 0; k < 2; ++k) dsW.emplace_back(new volScalarField("ds", mesh, N));
    dvW.emplace_back(new volVectorField("dv", mesh, N));
    const residualsIO res = solver->solveDelta(sW, vW, sSrc, vSrc, dsW, dvW);

    std::ofstream out(argv[2], std::ios::binary);
    auto put = [&](double v) { out.write(reinterpret_cast<const char*>(&v), sizeof v); };
    for (int f = 0; f < F; ++f) put(phi.internal[f]);
    for (int i = 0; i < P; ++i)
      for (double v : phi.boundary[i]) put(v);
    for (int f = 0; f < F; ++f)
      for (int k = 0; k < 3; ++k) put(phiU.internal[f][k]);
    for (int i = 0; i < P; ++i)
      for (const vector& v : phiU.boundary[i])
        for (int k = 0; k < 3; ++k) put(v[k]);
    for (int f = 0; f < F; ++f) put(phiE.internal[f]);
    for (int i = 0; i < P; ++i)
      for (double v : phiE.boundary[i]) put(v);
    for (int c = 0; c < N; ++c) {
      put(dsW[0]->internal[c]);
      for (int k = 0; k < 3; ++k) put(dvW[0]->internal[c][k]);
      put(dsW[1]->internal[c]);
    }
    put(res.nIterations);
    put(res.initRes[0]);
    std::printf("scheme %s solver %s cycles %d\n", scheme->type().c_str(), argv[4], res.nIterations);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
