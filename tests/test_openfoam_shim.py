"""The OpenFOAM-side shim (icsfoam_gb300/openfoam/gb300GPU.C) compiled and run.

The shim registers AUSMPlusUpGPU / HLLCGPU / ROEGPU in convectiveFluxScheme's
selection table and GMRESGPU in coupledMatrix::solver's, and forwards to the
C ABI.  Without OpenFOAM it is compiled against minimal stand-ins of the
OpenFOAM and ICSFoam types (tests/openfoam_stubs) and driven like dbnsFoam
drives the reference: the driver selects the scheme and the solver by name
from dictionaries, calls calcFlux and solveDelta on a case written by this
test.  On the CPU the shim is linked to the oracle (the icsref_ prefix) and
its fluxes and increment must equal the oracle's own entry points on the
same state (fluxes 1e-12, increment 1e-10, equal GMRES cycles); on the GPU
it is linked to the CUDA library and must match the oracle the same way.
"""

import os
import struct
import subprocess

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases

from test_gpu_parity import perturb, relerr  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUBS = os.path.join(ROOT, "tests", "openfoam_stubs")
SHIM = os.path.join(ROOT, "icsfoam_gb300", "openfoam")


def _compile(out, oracle):
    from icsfoam_gb300 import _build

    import oracle as oracle_pkg

    srcs = [os.path.join(STUBS, "shim_driver.C"), os.path.join(SHIM, "gb300GPU.C")]
    inc = ["-I" + STUBS, "-I" + SHIM, "-I" + os.path.join(ROOT, "include")]
    if oracle:
        libdir = os.path.dirname(oracle_pkg.build.build())
        extra = ["-include", os.path.join(STUBS, "oracle_prefix.H"), "-L" + libdir, "-licsref"]
    else:
        if not os.path.exists(_build.GPU_LIB):
            pytest.skip("CUDA library not built")
        libdir = os.path.dirname(_build.GPU_LIB)
        extra = ["-L" + libdir, "-licsgpu"]
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror"] + inc + srcs + ["-o", out] + extra + \
          ["-Wl,-rpath," + libdir]
    subprocess.check_call(cmd)
    return out


def _case(binding, tmp_path, flux):
    """The workload, its oracle reference results and the case file for the driver."""
    w = perturb(cases.bump_channel(24, 8, 4, ordering_mode="colour", flux=flux))
    m = w.mesh
    h = abi.CaseHandle(binding, m, cases.make_config(binding, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    bs = h.get_boundary_state()
    ref = {"flux": h.calc_flux()}
    h.residual()
    h.assemble_jacobian()
    perf, dW, _ = h.solve_increment()
    ref["dW"], ref["cycles"] = dW, perf.n_iterations
    R, Cp = w.settings["R"], w.settings["Cp"]
    st = h.get_state()
    path = str(tmp_path / ("case_%s.bin" % flux))
    with open(path, "wb") as f:
        wr = lambda a, t="d": f.write(np.ascontiguousarray(a, dtype=np.float64 if t == "d" else np.int32).tobytes())
        f.write(struct.pack("<iii", m.n_cells, m.n_faces, len(m.patches)))
        f.write(struct.pack("<dd", R, Cp))
        wr(m.owner, "i")
        wr(m.neighbour, "i")
        for a in (m.Sf, m.Cf, m.weights, m.delta_coeffs, m.nonorth_delta_coeffs, m.C, m.V):
            wr(a)
        for pi, p in enumerate(m.patches):
            sel = m.b_patch == pi
            f.write(p.name.encode().ljust(32, b"\0"))
            f.write((b"wall" if p.is_wall else b"patch").ljust(32, b"\0"))
            f.write(struct.pack("<i", p.kind))
            f.write(struct.pack("<7d", p.p, p.T, *p.U, p.p0, p.T0))
            f.write(struct.pack("<i", int(sel.sum())))
            wr(m.b_cell[sel], "i")
            wr(m.b_Sf[sel])
            wr(m.b_Cf[sel])
            wr(m.b_delta_coeffs[sel])
        rho = st["W"][:, 0]
        wr(rho)
        wr(st["U"])
        wr(st["p"])
        wr(st["T"])
        for pi in range(len(m.patches)):
            sel = m.b_patch == pi
            wr(bs["p"][sel] / (R * bs["T"][sel]))
            wr(bs["U"][sel])
            wr(bs["p"][sel])
            wr(bs["T"][sel])
    return w, ref, path


def _run(exe, case, out, flux):
    subprocess.run([exe, case, out, flux + "GPU", "GMRESGPU"], check=True, capture_output=True, text=True)
    return np.fromfile(out, dtype=np.float64)


def _compare(w, ref, got):
    FB = w.mesh.n_faces + w.mesh.n_bfaces
    N = w.mesh.n_cells
    phi, phiU, phiE = got[:FB], got[FB:4 * FB].reshape(FB, 3), got[4 * FB:5 * FB]
    dW = got[5 * FB:5 * FB + 5 * N].reshape(N, 5)
    cycles = int(got[5 * FB + 5 * N])
    fo = ref["flux"]
    assert relerr(phi, fo[0]) < 1e-12
    assert relerr(phiU, fo[1]) < 1e-12
    assert relerr(phiE, fo[2]) < 1e-12
    assert cycles == ref["cycles"]
    assert relerr(dW, ref["dW"]) < 1e-10


@pytest.mark.parametrize("flux", ["HLLC", "AUSMPlusUp", "ROE"])
def test_shim_selected_by_name_matches_the_oracle(oracle_binding, tmp_path, flux):
    exe = _compile(str(tmp_path / "shim_ref"), oracle=True)
    w, ref, case = _case(oracle_binding, tmp_path, flux)
    _compare(w, ref, _run(exe, case, str(tmp_path / "out.bin"), flux))


def test_shim_refuses_unknown_names(tmp_path, oracle_binding):
    exe = _compile(str(tmp_path / "shim_ref"), oracle=True)
    w, ref, case = _case(oracle_binding, tmp_path, "HLLC")
    r = subprocess.run([exe, case, str(tmp_path / "o.bin"), "UpwindGPU", "GMRESGPU"], capture_output=True, text=True)
    assert r.returncode != 0 and "Unknown convectiveFluxScheme" in r.stderr
    r = subprocess.run([exe, case, str(tmp_path / "o.bin"), "HLLCGPU", "BiCGGPU"], capture_output=True, text=True)
    assert r.returncode != 0 and "Unknown solver" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("flux", ["HLLC", "AUSMPlusUp"])
def test_shim_on_the_gpu_matches_the_oracle(oracle_binding, tmp_path, flux):
    exe = _compile(str(tmp_path / "shim_gpu"), oracle=False)
    w, ref, case = _case(oracle_binding, tmp_path, flux)
    _compare(w, ref, _run(exe, case, str(tmp_path / "out.bin"), flux))
