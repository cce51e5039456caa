"""OpenFOAM case input/output for the hot path: polyMesh, initial fields and
the dictionaries that select the schemes.

``load_case(path)`` reads an ASCII OpenFOAM case the way dbnsFoam starts
from one -- ``constant/polyMesh/{points,faces,owner,neighbour,boundary}``,
``0/{p,U,T}``, ``constant/thermophysicalProperties``, ``system/{fvSchemes,
fvSolution,controlDict}`` -- and returns the mesh (geometry computed here,
see ``mesh.py``), the cell fields and an ``ics_config``-compatible settings
dict, ready for ``abi.CaseHandle`` or ``schemes.Case``.  ``write_case``
writes a mesh and fields back as an ASCII case (polyMesh + 0/ fields), so a
generated case can be inspected or run by OpenFOAM.

The boundary conditions of the three fields are folded into the patch kinds
the C ABI implements:

==============================================  ==========================
p / U / T boundary types                        patch kind
==============================================  ==========================
empty                                           dropped (empty direction)
fixedValue / fixedValue / fixedValue            FIXED (values taken)
zeroGradient / zeroGradient|inletOutlet / same  ZERO_GRADIENT
zeroGradient / slip|symmetry(Plane) / zeroGr.   SLIP
fixedValue / zeroGradient|inletOutlet|pIOV /    PRESSURE_OUTLET
   zeroGradient|inletOutlet
totalPressure / pressureInletOutletVelocity /   TOTAL_INLET (p0, T0)
   totalTemperature
zeroGradient / noSlip|fixedValue 0 / fixedValue ISOTHERMAL_WALL
cyclic / cyclic / cyclic (cyclic polyPatch)     CYCLIC (neighbourPatch, transform)
==============================================  ==========================

``inletOutlet`` is taken as zeroGradient (outflow).  Other combinations,
non-uniform boundary values, cyclicAMI and processor patches and binary
files raise ``ValueError``.  Only ASCII format is read.

Moving reference frames: when ``constant/MRFProperties`` or
``constant/MRFTranslatingProperties`` exists, its zones are built on the
cell zones of ``constant/polyMesh/cellZones`` (in the returned, possibly
renumbered, cell order) and returned as ``dicts["mrf_zones"]`` = (rotating,
translating), ready for ``mrf.frame_fields``; ``write_mrf`` writes them.
"""

from __future__ import annotations

import os
import re
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import mesh as M
from . import ordering

RR = 8314.46261815324  # universal gas constant [J/(kmol K)] (OpenFOAM thermodynamics::RR)


# ------------------------------------------------------------------ parsing
def _tokens(text: str) -> List[str]:
    """OpenFOAM tokens: punctuation, quoted strings and words; a word keeps an
    attached balanced parenthesised part (``reconstruct(rho)``, ``div(phi,U)``)."""
    out = []
    i, n = 0, len(text)
    while i < n:
        ch = text[i]
        if ch.isspace():
            i += 1
        elif ch in "{};[]()":
            out.append(ch)
            i += 1
        elif ch == '"':
            j = text.index('"', i + 1)
            out.append(text[i:j + 1])
            i = j + 1
        else:
            j = i
            depth = 0
            while j < n:
                c = text[j]
                if c == "(":
                    depth += 1
                elif c == ")":
                    if depth == 0:
                        break
                    depth -= 1
                elif depth == 0 and (c.isspace() or c in "{};[]\""):
                    break
                j += 1
            out.append(text[i:j])
            i = j
    return out


def _strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def parse_dict(text: str) -> Dict:
    """Parse an OpenFOAM dictionary into nested dicts.

    Keyword entries become ``key: "tok tok ..."`` (tokens joined by single
    spaces, parentheses kept as tokens), sub-dictionaries become dicts.
    ``$name`` references to earlier top-level entries are substituted;
    ``#`` directives are ignored.
    """
    toks = _tokens(_strip_comments(text))
    pos = 0

    def parse_block(end: Optional[str]) -> Dict:
        nonlocal pos
        out: Dict = {}
        while pos < len(toks):
            t = toks[pos]
            if end and t == end:
                pos += 1
                return out
            if t.startswith("#"):
                # directive: skip to end of line-like statement (its single argument)
                pos += 2
                continue
            key = t.strip('"')
            pos += 1
            if pos < len(toks) and toks[pos] == "{":
                pos += 1
                out[key] = parse_block("}")
                continue
            vals = []
            depth = 0
            while pos < len(toks):
                v = toks[pos]
                if v == ";" and depth == 0:
                    pos += 1
                    break
                if v in ("(", "["):
                    depth += 1
                elif v in (")", "]"):
                    depth -= 1
                vals.append(v)
                pos += 1
            s = " ".join(vals)
            if s.startswith("$") and s[1:] in out:
                s = out[s[1:]]
            out[key] = s
        return out

    return parse_block(None)


def _read(path: str) -> str:
    with open(path) as f:
        return f.read()


def _header_and_body(text: str) -> Tuple[Dict, str]:
    text = _strip_comments(text)
    m = re.search(r"FoamFile\s*\{(.*?)\}", text, flags=re.S)
    header = parse_dict(m.group(1)) if m else {}
    if header.get("format", "ascii") != "ascii":
        raise ValueError("only ASCII OpenFOAM files are supported")
    body = text[m.end():] if m else text
    return header, body


def _list_body(body: str) -> Tuple[int, str]:
    """Count and the inside of the top-level ``N ( ... )`` list of a file body."""
    m = re.search(r"(\d+)\s*\(", body)
    if not m:
        raise ValueError("no list found")
    n = int(m.group(1))
    start = m.end()
    end = body.rfind(")")
    return n, body[start:end]


def read_points(path: str) -> np.ndarray:
    _, body = _header_and_body(_read(path))
    n, inner = _list_body(body)
    v = np.array(re.findall(r"[-+0-9.eE]+", inner), dtype=np.float64)
    if v.size != 3 * n:
        raise ValueError("%s: expected %d points" % (path, n))
    return v.reshape(n, 3)


def read_faces(path: str):
    _, body = _header_and_body(_read(path))
    n, inner = _list_body(body)
    groups = re.findall(r"(\d+)\s*\(([^)]*)\)", inner)
    if len(groups) != n:
        raise ValueError("%s: expected %d faces" % (path, n))
    faces = [np.array(g[1].split(), dtype=np.int64) for g in groups]
    for f, g in zip(faces, groups):
        if len(f) != int(g[0]):
            raise ValueError("%s: face size mismatch" % path)
    return _pack_faces(faces)


def read_labels(path: str) -> np.ndarray:
    _, body = _header_and_body(_read(path))
    n, inner = _list_body(body)
    v = np.array(inner.split(), dtype=np.int64)
    if v.size != n:
        raise ValueError("%s: expected %d labels" % (path, n))
    return v


def read_boundary(path: str) -> List[Dict]:
    _, body = _header_and_body(_read(path))
    n, inner = _list_body(body)
    d = parse_dict(inner)
    out = []
    for name, e in d.items():
        if not isinstance(e, dict):
            continue
        out.append({"name": name, "type": e.get("type", "patch"), "nFaces": int(e["nFaces"]),
                    "startFace": int(e["startFace"]), "dict": e})
    if len(out) != n:
        raise ValueError("%s: expected %d patches" % (path, n))
    return out


def _pack_faces(faces: List[np.ndarray]):
    """(n, k) int array when every face has k points, else an object array."""
    if faces and all(len(f) == len(faces[0]) for f in faces):
        return np.stack(faces).astype(np.int64)
    arr = np.empty(len(faces), dtype=object)
    for i, f in enumerate(faces):
        arr[i] = f
    return arr


def _parse_value(s: str, n_comp: int):
    """'uniform X' / 'uniform (x y z)' -> ndarray(n_comp,); 'nonuniform List<..> N (...)' -> (N, n_comp)."""
    s = s.strip()
    if s.startswith("uniform"):
        nums = re.findall(r"[-+0-9.eE]+", s[len("uniform"):])
        v = np.array(nums, dtype=np.float64)
        if v.size != n_comp:
            raise ValueError("bad uniform value %r" % s)
        return v
    if s.startswith("nonuniform"):
        m = re.search(r"(\d+)\s*\(", s)
        n = int(m.group(1))
        inner = s[m.end():s.rfind(")")]
        v = np.array(re.findall(r"[-+0-9.eE]+", inner), dtype=np.float64)
        if v.size != n * n_comp:
            raise ValueError("bad nonuniform list")
        return v.reshape(n, n_comp)
    raise ValueError("unsupported field value %r" % s)


def read_field(path: str, n_comp: int) -> Tuple[np.ndarray, Dict]:
    header, body = _header_and_body(_read(path))
    d = parse_dict(body)
    internal = _parse_value(d["internalField"], n_comp)
    return internal, d.get("boundaryField", {})


# ----------------------------------------------------------- patch kinds
_ZG = ("zeroGradient", "inletOutlet")
_SYM = ("slip", "symmetryPlane", "symmetry")


def _uval(e: Dict, key: str, n_comp: int):
    if key not in e:
        raise ValueError("boundary entry needs %r" % key)
    v = _parse_value(e[key], n_comp)
    if v.ndim != 1:
        raise ValueError("non-uniform boundary values are not supported")
    return v


def patch_from_bcs(name: str, ptype: str, bp: Dict, bU: Dict, bT: Dict, bdict: Optional[Dict] = None) -> M.Patch:
    """Fold the p, U, T boundary conditions of one patch into a patch kind.

    A ``cyclic`` polyPatch (with cyclic p, U, T) becomes a coupled patch; its
    transform (``bdict``: neighbourPatch, transform translational /
    rotational, separationVector or rotationAxis / rotationCentre /
    rotationAngle) is resolved against the face geometry by
    ``mesh_from_polymesh``.
    """
    tp, tU, tT = bp.get("type"), bU.get("type"), bT.get("type")
    is_wall = ptype == "wall"
    if ptype == "empty" or "empty" in (tp, tU, tT):
        return M.Patch(name, M.PATCH_EMPTY)
    if ptype == "cyclic":
        if any(t not in (None, "cyclic") for t in (tp, tU, tT)):
            raise ValueError("patch %s: a cyclic patch needs cyclic p, U and T" % name)
        d = bdict or {}
        if "neighbourPatch" not in d:
            raise ValueError("patch %s: cyclic without neighbourPatch" % name)
        q = M.Patch(name, M.PATCH_CYCLIC, partner=d["neighbourPatch"])
        q.transform = d  # resolved in mesh_from_polymesh
        q.match_tolerance = float(d.get("matchTolerance", 1e-4))
        return q
    if ptype in ("cyclicAMI", "processor") or "cyclic" in (tp, tU, tT):
        raise ValueError("patch %s: %s patches are not supported" % (name, ptype))
    if tp == "fixedValue" and tU == "fixedValue" and tT == "fixedValue":
        U = _uval(bU, "value", 3)
        if is_wall and np.all(U == 0):
            raise ValueError("patch %s: fixed-pressure walls are not supported" % name)
        return M.Patch(name, M.PATCH_FIXED, is_wall=is_wall, p=float(_uval(bp, "value", 1)[0]),
                       T=float(_uval(bT, "value", 1)[0]), U=tuple(U))
    if tp == "zeroGradient" and tU in _SYM and tT in _ZG + ("symmetryPlane", "symmetry"):
        return M.Patch(name, M.PATCH_SLIP, is_wall=is_wall)
    if tp in ("symmetryPlane", "symmetry") and tU in ("symmetryPlane", "symmetry"):
        return M.Patch(name, M.PATCH_SLIP, is_wall=is_wall)
    if tp == "zeroGradient" and tU in _ZG and tT in _ZG:
        return M.Patch(name, M.PATCH_ZERO_GRADIENT, is_wall=is_wall)
    if tp == "fixedValue" and tU in _ZG + ("pressureInletOutletVelocity",) and tT in _ZG:
        return M.Patch(name, M.PATCH_PRESSURE_OUTLET, is_wall=is_wall, p=float(_uval(bp, "value", 1)[0]))
    if tp == "totalPressure" and tU == "pressureInletOutletVelocity" and tT == "totalTemperature":
        return M.Patch(name, M.PATCH_TOTAL_INLET, is_wall=is_wall, p0=float(_uval(bp, "p0", 1)[0]),
                       T0=float(_uval(bT, "T0", 1)[0]))
    if tp == "zeroGradient" and tT == "fixedValue" and (
            tU == "noSlip" or (tU == "fixedValue" and np.all(_uval(bU, "value", 3) == 0))):
        return M.Patch(name, M.PATCH_ISOTHERMAL_WALL, is_wall=True, T=float(_uval(bT, "value", 1)[0]))
    raise ValueError("patch %s: unsupported boundary conditions p=%s U=%s T=%s" % (name, tp, tU, tT))


# ------------------------------------------------------------------ mesh
def _vec3(s) -> np.ndarray:
    v = np.array(str(s).replace("(", " ").replace(")", " ").split(), dtype=np.float64)
    if v.size != 3:
        raise ValueError("expected a vector, got %r" % s)
    return v


def _resolve_cyclic(patches: List[M.Patch], centres: Dict[str, np.ndarray]):
    """Rotation and separation of each cyclic pair from its transform entry
    (OpenFOAM cyclicTransform): translational - separationVector (this patch
    to its neighbour); rotational - rotationAxis, rotationCentre and
    rotationAngle, the sign that maps the neighbour's face centres onto this
    patch's being taken; no transform - the translation between the patch
    centroids.  The face pairing is checked again when the mesh is built."""
    by = {p.name: p for p in patches}
    for p in patches:
        if p.kind != M.PATCH_CYCLIC:
            continue
        d = getattr(p, "transform", {}) or {}
        ca, cb = centres[p.name], centres[p.partner]
        kind = d.get("transform", "")
        if kind == "rotational":
            axis = _vec3(d["rotationAxis"])
            ctr = _vec3(d.get("rotationCentre", "(0 0 0)"))
            ang = float(d["rotationAngle"])
            best = None
            for a in (ang, -ang):
                R = M.rotation_matrix(axis, a)
                err = np.abs((cb - ctr) @ R.T + ctr - ca).max() if len(ca) else 0.0
                if best is None or err < best[0]:
                    best = (err, R)
            p.rotation, p.centre, p.separation = tuple(best[1].ravel()), tuple(ctr), (0.0, 0.0, 0.0)
        else:
            if kind == "translational":
                sep = -_vec3(d["separationVector"])
            else:
                sep = (ca.mean(axis=0) - cb.mean(axis=0)) if len(ca) else np.zeros(3)
            p.rotation, p.separation = tuple(np.eye(3).ravel()), tuple(sep)
        if by[p.partner].partner != p.name:
            raise ValueError("cyclic patches %s and %s do not name each other" % (p.name, p.partner))


def mesh_from_polymesh(points, faces, owner, neighbour, boundary: List[Dict], patches: List[M.Patch]) -> M.Mesh:
    centres = {}
    for b, p in zip(boundary, patches):
        if p.kind == M.PATCH_CYCLIC:
            sl = slice(b["startFace"], b["startFace"] + b["nFaces"])
            centres[p.name] = M.face_centres_and_areas(points, faces[sl])[0] if b["nFaces"] else np.zeros((0, 3))
    _resolve_cyclic(patches, centres)
    nInt = len(neighbour)
    own = owner[:nInt].astype(np.int64)
    nei = neighbour.astype(np.int64)
    fp_int = faces[:nInt]
    entries = []
    by_name = {p.name: p for p in patches}
    for b in boundary:
        sl = slice(b["startFace"], b["startFace"] + b["nFaces"])
        entries.append((by_name[b["name"]], faces[sl], owner[sl].astype(np.int64)))
    plist = [by_name[b["name"]] for b in boundary]
    return M._finish(points, fp_int, own, nei, entries, plist)


def read_cell_zones(path: str) -> Dict[str, np.ndarray]:
    """constant/polyMesh/cellZones: {name: cell labels}."""
    _, body = _header_and_body(_read(path))
    n, inner = _list_body(body)
    zones: Dict[str, np.ndarray] = {}
    pos = 0
    for m in re.finditer(r"(\S+)\s*\{", inner):
        if m.start() < pos:
            continue
        depth, i = 1, m.end()
        while depth and i < len(inner):
            depth += {"{": 1, "}": -1}.get(inner[i], 0)
            i += 1
        block = inner[m.end():i - 1]
        pos = i
        lab = re.search(r"cellLabels\s+List<label>\s*(\d+)\s*(\{\s*(-?\d+)\s*\}|\(([^)]*)\))", block)
        if not lab:
            raise ValueError("%s: zone %s has no cellLabels" % (path, m.group(1)))
        cnt = int(lab.group(1))
        if lab.group(3) is not None:
            v = np.full(cnt, int(lab.group(3)), np.int64)
        else:
            v = np.array(lab.group(4).split(), dtype=np.int64)
        if v.size != cnt:
            raise ValueError("%s: zone %s: expected %d labels" % (path, m.group(1), cnt))
        zones[m.group(1)] = v
    if len(zones) != n:
        raise ValueError("%s: expected %d zones" % (path, n))
    return zones


def _time_dir(path: str, time: str) -> str:
    for cand in (time, time + ".orig"):
        d = os.path.join(path, cand)
        if os.path.isdir(d):
            return d
    raise FileNotFoundError(os.path.join(path, time))


def load_case(path: str, time: str = "0", ordering_mode: Optional[str] = None):
    """Read an ASCII OpenFOAM case; returns (mesh, fields, settings, dicts).

    fields = {"p": [N], "U": [N, 3], "T": [N]} in the (possibly renumbered)
    cell order; settings = ics_config field overrides for ``cases.make_config``;
    dicts = the parsed fvSchemes / fvSolution / thermophysicalProperties.
    """
    pm = os.path.join(path, "constant", "polyMesh")
    points = read_points(os.path.join(pm, "points"))
    faces = read_faces(os.path.join(pm, "faces"))
    owner = read_labels(os.path.join(pm, "owner"))
    neighbour = read_labels(os.path.join(pm, "neighbour"))
    boundary = read_boundary(os.path.join(pm, "boundary"))
    tdir = _time_dir(path, time)
    p_in, p_b = read_field(os.path.join(tdir, "p"), 1)
    U_in, U_b = read_field(os.path.join(tdir, "U"), 3)
    T_in, T_b = read_field(os.path.join(tdir, "T"), 1)
    patches = [patch_from_bcs(b["name"], b["type"], p_b.get(b["name"], {}), U_b.get(b["name"], {}),
                              T_b.get(b["name"], {}), b["dict"]) for b in boundary]
    mesh = mesh_from_polymesh(points, faces, owner, neighbour, boundary, patches)
    N = mesh.n_cells
    p = np.broadcast_to(p_in.reshape(-1), (N,)).copy() if p_in.ndim == 1 else p_in[:, 0].copy()
    T = np.broadcast_to(T_in.reshape(-1), (N,)).copy() if T_in.ndim == 1 else T_in[:, 0].copy()
    U = np.broadcast_to(U_in, (N, 3)).copy()
    old_to_new = np.arange(N)
    if ordering_mode:
        perm = ordering.permutation(mesh, ordering_mode)
        mesh = M.renumber(mesh, perm)
        p, U, T = p[perm], U[perm], T[perm]
        old_to_new = np.empty(N, np.int64)
        old_to_new[perm] = np.arange(N)
    dicts = {}
    for name, sub in (("fvSchemes", "system"), ("fvSolution", "system"), ("controlDict", "system"),
                      ("thermophysicalProperties", "constant"), ("MRFProperties", "constant"),
                      ("MRFTranslatingProperties", "constant")):
        f = os.path.join(path, sub, name)
        dicts[name] = parse_dict(_header_and_body(_read(f))[1]) if os.path.exists(f) else {}
    if dicts["MRFProperties"] or dicts["MRFTranslatingProperties"]:
        from . import mrf as MRF
        zf = os.path.join(pm, "cellZones")
        cz = read_cell_zones(zf) if os.path.exists(zf) else {}
        cz = {k: old_to_new[v] for k, v in cz.items()}
        dicts["mrf_zones"] = MRF.zones_from_dicts(dicts["MRFProperties"], dicts["MRFTranslatingProperties"], cz)
    settings = settings_from_dicts(dicts)
    return mesh, {"p": p, "U": U, "T": T}, settings, dicts


def thermo_from_dict(tp: Dict) -> Dict:
    mix = tp.get("mixture", {})
    out = {}
    mw = mix.get("specie", {}).get("molWeight")
    if mw is not None:
        out["R"] = RR / float(mw)
    cp = mix.get("thermodynamics", {}).get("Cp")
    if cp is not None:
        out["Cp"] = float(cp)
    tr = mix.get("transport", {})
    ttype = tp.get("thermoType", {}).get("transport", "const")
    if ttype == "sutherland":
        out["sutherland"] = 1
        out["As"] = float(tr["As"])
        out["Ts"] = float(tr["Ts"])
        out["viscous"] = 1
    elif "mu" in tr and float(tr["mu"]) > 0:
        out["mu"] = float(tr["mu"])
        out["viscous"] = 1
    if "Pr" in tr:
        out["Pr"] = float(tr["Pr"])
    return out


def settings_from_dicts(dicts: Dict) -> Dict:
    """ics_config overrides from the case dictionaries (through schemes.config_from_dicts)."""
    from . import schemes

    class _Rec:  # records attribute assignments like a ctypes Config
        def __init__(self):
            self.__dict__["vals"] = {}

        def __setattr__(self, k, v):
            self.vals[k] = v

    class _B:
        def default_config(self):
            return _Rec()

    rec = schemes.config_from_dicts(_B(), dicts.get("fvSchemes", {}), dicts.get("fvSolution", {}),
                                    None)
    out = dict(rec.vals)
    out.update(thermo_from_dict(dicts.get("thermophysicalProperties", {})))
    dt = dicts.get("controlDict", {}).get("deltaT")
    if dt is not None:
        out["delta_t"] = float(dt)
    return out


# ------------------------------------------------------------------ writing
_HEADER = """/*--------------------------------*- C++ -*----------------------------------*\\
  written by icsfoam_gb300.foam_case
\\*---------------------------------------------------------------------------*/
FoamFile
{
    version     2.0;
    format      ascii;
    class       %s;
    location    "%s";
    object      %s;
}
"""


def _write(path: str, cls: str, loc: str, obj: str, body: str):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write(_HEADER % (cls, loc, obj))
        f.write(body)


def _faces_text(faces) -> List[str]:
    return ["%d(%s)" % (len(f), " ".join(str(int(x)) for x in f)) for f in faces]


def _transform_text(patch: M.Patch) -> str:
    """The cyclicTransform entries of a coupled patch (axis-angle from R)."""
    R = np.asarray(patch.rotation if patch.rotation is not None else np.eye(3).ravel(), np.float64).reshape(3, 3)
    ang = np.degrees(np.arccos(np.clip((np.trace(R) - 1.0) / 2.0, -1.0, 1.0)))
    if ang < 1e-12:
        sep = -np.asarray(patch.separation, np.float64)
        return "\n        transform translational;\n        separationVector (%.17g %.17g %.17g);" % tuple(sep)
    ax = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    ax = ax / np.linalg.norm(ax)
    return ("\n        transform rotational;\n        rotationAxis (%.17g %.17g %.17g);"
            "\n        rotationCentre (%.17g %.17g %.17g);\n        rotationAngle %.17g;"
            % (tuple(ax) + tuple(patch.centre) + (ang,)))


def write_case(path: str, mesh: M.Mesh, p: np.ndarray, U: np.ndarray, T: np.ndarray):
    """Write ``mesh`` and the cell fields as an ASCII case (polyMesh + 0/{p,U,T}).

    Boundary conditions are written back per patch kind (the inverse of the
    table in the module docstring); the mesh must carry its face points.
    """
    if mesh.points is None or mesh.face_points is None:
        raise ValueError("mesh has no point/face topology to write")
    pm = os.path.join(path, "constant", "polyMesh")
    F = mesh.n_faces
    faces = list(mesh.face_points) + list(mesh.b_face_points)
    owner = list(mesh.owner) + list(mesh.b_cell)
    boundary = []
    start = F
    for pi, patch in enumerate(mesh.patches):
        n = int(np.sum(mesh.b_patch == pi))
        boundary.append((patch, n, start))
        start += n
    # boundary faces are stored patch by patch already (b_patch sorted)
    if np.any(np.diff(mesh.b_patch) < 0):
        raise ValueError("boundary faces must be grouped by patch")
    e_fp, e_cell = getattr(mesh, "_empty", (np.zeros((0, 4), np.int64), np.zeros(0, np.int64)))
    if len(e_fp):
        faces += list(e_fp)
        owner += list(e_cell)
        boundary.append((M.Patch("emptyFaces", M.PATCH_EMPTY), len(e_fp), start))
    pts = "\n".join("(%.17g %.17g %.17g)" % tuple(x) for x in mesh.points)
    _write(os.path.join(pm, "points"), "vectorField", "constant/polyMesh", "points",
           "\n%d\n(\n%s\n)\n" % (len(mesh.points), pts))
    _write(os.path.join(pm, "faces"), "faceList", "constant/polyMesh", "faces",
           "\n%d\n(\n%s\n)\n" % (len(faces), "\n".join(_faces_text(faces))))
    _write(os.path.join(pm, "owner"), "labelList", "constant/polyMesh", "owner",
           "\n%d\n(\n%s\n)\n" % (len(owner), "\n".join(str(int(x)) for x in owner)))
    _write(os.path.join(pm, "neighbour"), "labelList", "constant/polyMesh", "neighbour",
           "\n%d\n(\n%s\n)\n" % (F, "\n".join(str(int(x)) for x in mesh.neighbour)))
    bl = []
    for patch, n, st in boundary:
        ptype = "empty" if patch.kind == M.PATCH_EMPTY else ("wall" if patch.is_wall else "patch")
        extra = ""
        if patch.kind == M.PATCH_CYCLIC:
            ptype = "cyclic"
            extra = "\n        neighbourPatch %s;" % patch.partner + _transform_text(patch)
        bl.append("    %s\n    {\n        type %s;\n        nFaces %d;\n        startFace %d;%s\n    }"
                  % (patch.name, ptype, n, st, extra))
    _write(os.path.join(pm, "boundary"), "polyBoundaryMesh", "constant/polyMesh", "boundary",
           "\n%d\n(\n%s\n)\n" % (len(boundary), "\n".join(bl)))

    def bc(patch):
        k = patch.kind
        u = "uniform (%.17g %.17g %.17g)" % tuple(patch.U)
        if k == M.PATCH_EMPTY:
            return ("empty", None), ("empty", None), ("empty", None)
        if k == M.PATCH_FIXED:
            return (("fixedValue", "value uniform %.17g" % patch.p), ("fixedValue", "value " + u),
                    ("fixedValue", "value uniform %.17g" % patch.T))
        if k == M.PATCH_SLIP:
            return ("zeroGradient", None), ("slip", None), ("zeroGradient", None)
        if k == M.PATCH_ZERO_GRADIENT:
            return ("zeroGradient", None), ("zeroGradient", None), ("zeroGradient", None)
        if k == M.PATCH_PRESSURE_OUTLET:
            return ("fixedValue", "value uniform %.17g" % patch.p), ("zeroGradient", None), ("zeroGradient", None)
        if k == M.PATCH_TOTAL_INLET:
            return (("totalPressure", "p0 uniform %.17g" % patch.p0), ("pressureInletOutletVelocity", None),
                    ("totalTemperature", "T0 uniform %.17g" % patch.T0))
        if k == M.PATCH_ISOTHERMAL_WALL:
            return ("zeroGradient", None), ("noSlip", None), ("fixedValue", "value uniform %.17g" % patch.T)
        if k == M.PATCH_CYCLIC:
            return ("cyclic", None), ("cyclic", None), ("cyclic", None)
        raise ValueError(patch.kind)

    def field(name, cls, values, idx, fmt):
        lines = ["\ndimensions [0 0 0 0 0 0 0];\n",
                 "internalField nonuniform List<%s> %d\n(\n%s\n);\n" % (
                     "vector" if cls == "volVectorField" else "scalar", len(values),
                     "\n".join(fmt(v) for v in values)),
                 "boundaryField\n{"]
        for patch, _, _ in boundary:
            t, extra = bc(patch)[idx]
            lines.append("    %s\n    {\n        type %s;%s\n    }" % (
                patch.name, t, ("\n        %s;" % extra) if extra else ""))
        lines.append("}\n")
        _write(os.path.join(path, "0", name), cls, "0", name, "\n".join(lines))

    field("p", "volScalarField", p, 0, lambda v: "%.17g" % v)
    field("U", "volVectorField", U, 1, lambda v: "(%.17g %.17g %.17g)" % tuple(v))
    field("T", "volScalarField", T, 2, lambda v: "%.17g" % v)


def write_mrf(path: str, mesh: M.Mesh, rotating=(), translating=()):
    """Write the zones as constant/polyMesh/cellZones (one zone per MRF zone,
    named zone0, zone1, ...) and constant/MRFProperties /
    constant/MRFTranslatingProperties (one sub-dictionary per zone)."""
    zones = list(rotating) + list(translating)
    blocks = []
    for i, z in enumerate(zones):
        c = np.asarray(z.cells)
        lab = np.nonzero(c)[0] if c.dtype == bool else np.sort(c.astype(np.int64))
        blocks.append("zone%d\n{\n    type cellZone;\n    cellLabels List<label> %d\n(\n%s\n)\n;\n}"
                      % (i, len(lab), "\n".join(str(int(x)) for x in lab)))
    _write(os.path.join(path, "constant", "polyMesh", "cellZones"), "regIOobject", "constant/polyMesh",
           "cellZones", "\n%d\n(\n%s\n)\n" % (len(zones), "\n".join(blocks)))
    vec = lambda v: "(%.17g %.17g %.17g)" % tuple(v)
    names = lambda ps: "(%s)" % " ".join(ps)
    rot = []
    for i, z in enumerate(rotating):
        rot.append("zone%d\n{\n    cellZone zone%d;\n    active %s;\n    nonRotatingPatches %s;\n"
                   "    origin %s;\n    axis %s;\n    omega %.17g;\n}" % (i, i, "yes" if z.active else "no",
                                                                       names(z.non_rotating_patches),
                                                                       vec(z.origin), vec(z.axis), z.omega))
    _write(os.path.join(path, "constant", "MRFProperties"), "dictionary", "constant", "MRFProperties",
           "\n" + "\n".join(rot) + "\n")
    tra = []
    for j, z in enumerate(translating):
        i = len(rotating) + j
        tra.append("zone%d\n{\n    cellZone zone%d;\n    active %s;\n    nonMovingPatches %s;\n"
                   "    frameVelocity %s;\n}" % (i, i, "yes" if z.active else "no", names(z.non_moving_patches),
                                                  vec(z.frame_velocity)))
    _write(os.path.join(path, "constant", "MRFTranslatingProperties"), "dictionary", "constant",
           "MRFTranslatingProperties", "\n" + "\n".join(tra) + "\n")
