"""Python front end of the CPU oracle (test infrastructure only).

This module is the oracle the GPU results are compared with.  Only the tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import it; the product package
``cc_abstemious_gb300`` never does.

It restates the input layer of cc_abstemious (serde's externally tagged JSON
of src/preprocess/input_data.rs:9-92, the frequency lists of src/tools.rs and
the per-frequency driver loop of src/analysis.rs:87-111) in Python and calls
the C restatement in ``bem_oracle.c`` for the numerics.
"""
import ctypes as C
import json
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build())
        _declare(_lib)
    return _lib


class OcProblem(C.Structure):
    _fields_ = [
        ("sound_speed", C.c_double), ("mass_density", C.c_double),
        ("problem_type", C.c_int32), ("method_type", C.c_int32), ("solver", C.c_int32),
        ("incident_type", C.c_int32), ("bc_type", C.c_int32), ("output_total", C.c_int32),
        ("output_pressure", C.c_int32), ("pad0", C.c_int32),
        ("tolerance", C.c_double), ("max_iterations", C.c_int64),
        ("incident_vec", C.c_double * 3), ("incident_amp", C.c_double * 2),
        ("bc_value", C.c_double * 2),
        ("hm_leaf", C.c_int64), ("hm_eta", C.c_double), ("hm_aca_tol", C.c_double),
        ("nfp", C.c_int64), ("field_points", C.c_void_p),
        ("n", C.c_int64), ("cpts", C.c_void_p),
        ("frequency", C.c_double),
    ]


class OcMesh(C.Structure):
    _fields_ = [
        ("nnodes", C.c_int64), ("nodes", C.POINTER(C.c_double)),
        ("nelem", C.c_int64), ("body", C.POINTER(C.c_int64)),
        ("etype", C.POINTER(C.c_int32)), ("conn_off", C.POINTER(C.c_int64)),
        ("conn", C.POINTER(C.c_int64)), ("nbodies", C.c_int64), ("status", C.c_int32),
    ]


class OcReport(C.Structure):
    _fields_ = [("num_mv", C.c_int64), ("restarts", C.c_int64), ("error", C.c_double),
                ("flag", C.c_int32), ("pad", C.c_int32)]


class OcBlockList(C.Structure):
    _fields_ = [("nblocks", C.c_int64), ("row_off", C.POINTER(C.c_int64)),
                ("rows", C.POINTER(C.c_int64)), ("col_off", C.POINTER(C.c_int64)),
                ("cols", C.POINTER(C.c_int64)), ("admissible", C.POINTER(C.c_int32)),
                ("root_diameter", C.c_double)]


class OcStdRng(C.Structure):
    _fields_ = [("key", C.c_uint32 * 8), ("counter", C.c_uint64),
                ("buf", C.c_uint32 * 64), ("idx", C.c_int32)]


ROWCOL_FN = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(C.c_int64), C.c_int64,
                        C.POINTER(C.c_int64), C.c_int64, C.POINTER(C.c_double))

_P = C.POINTER(OcProblem)
_vp = C.c_void_p
_i64 = C.c_int64
_d = C.c_double


def _declare(L):
    sig = {
        "oc_read_vtk": (C.c_int, [C.c_char_p, C.POINTER(OcMesh)]),
        "oc_mesh_free": (None, [C.POINTER(OcMesh)]),
        "oc_collocation": (_i64, [C.POINTER(OcMesh), _i64, _vp]),
        "oc_linspace": (C.c_int, [_d, _d, _i64, _vp]),
        "oc_logspace": (C.c_int, [_d, _d, _i64, _vp]),
        "oc_greens": (None, [_d, _vp, _vp, _vp, _vp, C.c_int, _vp, _vp]),
        "oc_gh": (None, [_P, _i64, _i64, _vp, _vp]),
        "oc_dense_surface": (None, [_P, _vp, _vp, _i64, C.c_int]),
        "oc_dense_field": (None, [_P, _vp, _vp, _i64]),
        "oc_lhs_factors": (None, [_P, _vp, _vp]),
        "oc_rhs_factors": (None, [_P, _vp, _vp]),
        "oc_row_or_column": (C.c_int, [_P, _vp, _i64, _vp, _i64, C.c_int, _vp]),
        "oc_incident_surface": (None, [_P, _vp]),
        "oc_incident_field": (None, [_P, _vp]),
        "oc_lu_solve": (C.c_int, [_i64, _vp, _i64, _vp]),
        "oc_gmres_dense": (C.c_int, [_i64, _vp, _i64, _i64, _d, _vp, C.POINTER(OcReport)]),
        "oc_solve_for_surface": (C.c_int, [_P, _vp, _vp, _vp, C.POINTER(OcReport), C.c_int]),
        "oc_get_field": (None, [_P, _vp, _vp, _i64, _vp, _vp, _vp, _vp]),
        "oc_convert_to_pressure": (None, [_P, _vp, _i64]),
        "oc_run_frequency": (C.c_int, [_P, _vp, _vp, _vp, _vp, C.POINTER(OcReport), C.c_int]),
        "oc_hmatrix_build": (_vp, [_i64, _vp, _i64, _i64, _d, _d, ROWCOL_FN, _vp]),
        "oc_hmatrix_free": (None, [_vp]),
        "oc_hmatrix_norm": (_d, [_vp]),
        "oc_hmatrix_gemv": (None, [_vp, _vp, _vp, _vp, _vp]),
        "oc_hmatrix_to_full": (None, [_vp, _vp, _i64]),
        "oc_hmatrix_stats": (None, [_vp, _vp]),
        "oc_hmatrix_num_blocks": (_i64, [_vp]),
        "oc_gmres_hmatrix": (C.c_int, [_vp, _i64, _d, _vp, C.POINTER(OcReport)]),
        "oc_block_list": (C.c_int, [_i64, _vp, _i64, _i64, _d, C.POINTER(OcBlockList)]),
        "oc_blocklist_free": (None, [C.POINTER(OcBlockList)]),
        "oc_block_tree_path_admissible": (C.c_int, [_i64, _vp, _i64, _i64, _d, _vp, C.c_int]),
        "oc_aca": (_i64, [_i64, _i64, _d, ROWCOL_FN, _vp, _vp, _vp, C.POINTER(C.c_double)]),
        "oc_stdrng_seed": (None, [C.POINTER(OcStdRng), C.c_uint64]),
        "oc_stdrng_u32": (C.c_uint32, [C.POINTER(OcStdRng)]),
        "oc_stdrng_u64": (C.c_uint64, [C.POINTER(OcStdRng)]),
        "oc_stdrng_f64": (_d, [C.POINTER(OcStdRng)]),
        "oc_uniform_usize_incl": (C.c_uint64, [C.POINTER(OcStdRng), C.c_uint64, C.c_uint64]),
        "oc_generate_random_ab": (None, [_i64, _i64, C.c_uint64, _vp, _vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _cbuf(n, m=None):
    return np.zeros((n,) if m is None else (n, m), dtype=np.complex128, order="F")


# --------------------------------------------------------------------------
# Input layer (input_data.rs:9-92, serde external tagging)
PROBLEM_TYPES = {"Interior": 0, "Exterior": 1}
METHOD_TYPES = {"Classical": 0, "BurtonMiller": 1}
SOLVERS = {"Direct": 0, "Iterative": 1, "Hierarchical": 2}
INCIDENT = {"PlaneWave": 0, "SphericalWave": 1}
BC_TYPES = {"Pressure": 0, "NormalVelocity": 1, "Impedance": 2}


def _tag(obj):
    if isinstance(obj, str):
        return obj, {}
    if not isinstance(obj, dict) or len(obj) != 1:
        raise ValueError("expected an externally tagged enum")
    (k, v), = obj.items()
    return k, v


def frequency_list(freq):
    """preprocess.rs:155-167 with tools.rs:1-24."""
    kind, v = _tag(freq)
    if kind == "List":
        return np.array(v["values"], dtype=float)
    n = int(v["number"])
    out = np.zeros(n)
    f = lib().oc_linspace if kind == "LinearSpaced" else lib().oc_logspace
    if kind not in ("LinearSpaced", "LogSpaced") or f(float(v["start"]), float(v["end"]), n, _ptr(out)):
        raise ValueError("bad frequency input")
    return out


class Mesh:
    """mesh_data.rs:96-175 through the C reader."""

    def __init__(self, path):
        self._m = OcMesh()
        st = lib().oc_read_vtk(os.fsencode(path), C.byref(self._m))
        if st:
            lib().oc_mesh_free(C.byref(self._m))
            raise ValueError(f"VTK read error {st} for {path}")
        self.nelem = self._m.nelem
        self.nnodes = self._m.nnodes
        self.nbodies = self._m.nbodies

    def collocation(self, body_index):
        n = lib().oc_collocation(C.byref(self._m), body_index, None)
        if n < 0:
            raise ValueError("bad element connectivity")
        out = np.zeros((n, 8))
        lib().oc_collocation(C.byref(self._m), body_index, _ptr(out))
        return out

    def __del__(self):
        try:
            lib().oc_mesh_free(C.byref(self._m))
        except Exception:
            pass


class Problem:
    """UserInput + PreData (preprocess.rs:24-124) for the oracle."""

    def __init__(self, inp, base_dir=None, cpts=None):
        self.input = inp
        mesh_file = inp["mesh_file"]
        if base_dir and not os.path.isabs(mesh_file):
            mesh_file = os.path.join(base_dir, mesh_file)
        self.body_index = int(inp["body_index"])
        if cpts is None:
            mesh = Mesh(mesh_file)
            if self.body_index < 1 or self.body_index > mesh.nbodies:
                raise ValueError("body_index out of range")
            cpts = mesh.collocation(self.body_index)
        self.cpts = np.ascontiguousarray(cpts, dtype=float)
        self.frequencies = frequency_list(inp["frequency"])
        s = OcProblem()
        s.sound_speed = float(inp["sound_speed"])
        s.mass_density = float(inp["mass_density"])
        s.problem_type = PROBLEM_TYPES[inp["problem_type"]]
        s.method_type = METHOD_TYPES[inp["method_type"]]
        kind, sv = _tag(inp["solver"])
        s.solver = SOLVERS[kind]
        s.tolerance = float(sv.get("tolerance", 0.0))
        s.max_iterations = int(sv.get("max_iterations", 0))
        # additive extension keys inside Hierarchical; defaults are the values
        # hard-coded in solve.rs:91-92, :119-120 and h_matrix.rs:136
        s.hm_leaf = int(sv.get("leaf_size", 32))
        s.hm_eta = float(sv.get("eta", 4.0))
        s.hm_aca_tol = float(sv.get("aca_tolerance", 1e-4))
        kind, iv = _tag(inp["incident_wave"])
        s.incident_type = INCIDENT[kind]
        vec = iv["direction"] if kind == "PlaneWave" else iv["origin"]
        for i in range(3):
            s.incident_vec[i] = float(vec[i])
        s.incident_amp[0], s.incident_amp[1] = map(float, iv["amplitude"])
        bc = inp["surface_bc"]
        s.bc_type = BC_TYPES[bc["bc_type"]]
        s.bc_value[0], s.bc_value[1] = map(float, bc["value"])
        out = inp["output"]
        s.output_total = 1 if out["o_type"] == "Total" else 0
        s.output_pressure = 1 if out["field"] == "Pressure" else 0
        self.field_points = np.ascontiguousarray(np.array(out["field_points"], dtype=float).reshape(-1, 3))
        s.nfp = len(self.field_points)
        s.field_points = _ptr(self.field_points)
        s.n = len(self.cpts)
        s.cpts = _ptr(self.cpts)
        self.s = s
        self.n = int(s.n)
        self.nfp = int(s.nfp)
        self.set_frequency_index(0)

    @classmethod
    def from_json(cls, text, base_dir=None):
        return cls(json.loads(text), base_dir)

    def set_frequency_index(self, i):
        self.ifreq = i
        self.s.frequency = float(self.frequencies[i]) if len(self.frequencies) else 0.0

    @property
    def p(self):
        return C.byref(self.s)

    @property
    def frequency(self):
        return self.s.frequency

    @property
    def wavenumber(self):
        return 2.0 * np.pi * self.s.frequency / self.s.sound_speed

    # -- influence_matrix.rs ---------------------------------------------
    def dense_surface(self, nthreads=1):
        H, G = _cbuf(self.n, self.n), _cbuf(self.n, self.n)
        lib().oc_dense_surface(self.p, _ptr(H), _ptr(G), self.n, nthreads)
        return H, G

    def dense_field(self):
        M, L = _cbuf(self.nfp, self.n), _cbuf(self.nfp, self.n)
        lib().oc_dense_field(self.p, _ptr(M), _ptr(L), self.nfp)
        return M, L

    def row_or_column(self, I, J, side):
        I = np.ascontiguousarray(I, dtype=np.int64)
        J = np.ascontiguousarray(J, dtype=np.int64)
        out = _cbuf(max(len(I), len(J)))
        if lib().oc_row_or_column(self.p, _ptr(I), len(I), _ptr(J), len(J), side, _ptr(out)):
            raise ValueError("i or j must be singleton")
        return out

    def lhs_factors(self):
        a, b = np.zeros(2), np.zeros(2)
        lib().oc_lhs_factors(self.p, _ptr(a), _ptr(b))
        return complex(*a), complex(*b)

    def rhs_factors(self):
        a, b = np.zeros(2), np.zeros(2)
        lib().oc_rhs_factors(self.p, _ptr(a), _ptr(b))
        return complex(*a), complex(*b)

    # -- incident_wave.rs --------------------------------------------------
    def incident_surface(self):
        out = _cbuf(self.n)
        lib().oc_incident_surface(self.p, _ptr(out))
        return out

    def incident_field(self):
        out = _cbuf(self.nfp)
        lib().oc_incident_field(self.p, _ptr(out))
        return out

    # -- solve.rs ----------------------------------------------------------
    def solve_for_surface(self, rhs_inc, nthreads=1):
        rhs_inc = np.ascontiguousarray(rhs_inc, dtype=np.complex128)
        phi, vn = _cbuf(self.n), _cbuf(self.n)
        rep = OcReport()
        st = lib().oc_solve_for_surface(self.p, _ptr(rhs_inc), _ptr(phi), _ptr(vn), C.byref(rep), nthreads)
        return phi, vn, st, rep

    def get_field(self, M, L, phi, vn, phi_inc_fp):
        out = _cbuf(self.nfp)
        M = np.asfortranarray(M, dtype=np.complex128)
        L = np.asfortranarray(L, dtype=np.complex128)
        lib().oc_get_field(self.p, _ptr(M), _ptr(L), self.nfp, _ptr(np.ascontiguousarray(phi)),
                           _ptr(np.ascontiguousarray(vn)), _ptr(np.ascontiguousarray(phi_inc_fp)), _ptr(out))
        return out

    def run_frequency(self, nthreads=1):
        phi, vn = _cbuf(self.n), _cbuf(self.n)
        fps, fpi = _cbuf(self.nfp), _cbuf(self.nfp)
        rep = OcReport()
        st = lib().oc_run_frequency(self.p, _ptr(phi), _ptr(vn), _ptr(fps), _ptr(fpi), C.byref(rep), nthreads)
        return dict(phi=phi, vn=vn, scattered=fps, incident=fpi, status=st, report=rep)

    def run(self, nthreads=1):
        """Analysis::run (analysis.rs:57-118) + convert_results (postprocess.rs:70-79)."""
        results = []
        for i in range(len(self.frequencies)):
            self.set_frequency_index(i)
            r = self.run_frequency(nthreads)
            if self.s.output_pressure:
                lib().oc_convert_to_pressure(self.p, _ptr(r["scattered"]), self.nfp)
                lib().oc_convert_to_pressure(self.p, _ptr(r["incident"]), self.nfp)
            r["frequency"] = float(self.frequencies[i])
            results.append(r)
        return results


# --------------------------------------------------------------------------
def greens(k, x, nx, y, ny, bm):
    g, h = np.zeros(2), np.zeros(2)
    arr = [np.ascontiguousarray(v, dtype=float) for v in (x, nx, y, ny)]
    lib().oc_greens(k, *[_ptr(a) for a in arr], int(bm), _ptr(g), _ptr(h))
    return complex(*g), complex(*h)


def lu_solve(A, b):
    A = np.asfortranarray(A, dtype=np.complex128)
    x = np.array(b, dtype=np.complex128)
    st = lib().oc_lu_solve(A.shape[0], _ptr(A), A.shape[0], _ptr(x))
    return x, st


def gmres_dense(A, b, max_it, tol):
    A = np.asfortranarray(A, dtype=np.complex128)
    x = np.array(b, dtype=np.complex128)
    rep = OcReport()
    st = lib().oc_gmres_dense(A.shape[0], _ptr(A), A.shape[0], max_it, tol, _ptr(x), C.byref(rep))
    return x, st, rep


def generate_random_ab(m, n, seed):
    """solve.rs:194-209 through the rand 0.9 StdRng restatement."""
    A = _cbuf(m, n)
    b = _cbuf(n)
    lib().oc_generate_random_ab(m, n, seed, _ptr(A), _ptr(b))
    return A, b


class StdRng:
    def __init__(self, seed):
        self.r = OcStdRng()
        lib().oc_stdrng_seed(C.byref(self.r), seed)

    def u32(self):
        return lib().oc_stdrng_u32(C.byref(self.r))

    def u64(self):
        return lib().oc_stdrng_u64(C.byref(self.r))

    def f64(self):
        return lib().oc_stdrng_f64(C.byref(self.r))

    def uniform_incl(self, lo, hi):
        return lib().oc_uniform_usize_incl(C.byref(self.r), lo, hi)


def _matrix_gen(A):
    A = np.asfortranarray(A, dtype=np.complex128)

    def gen(ctx, I, ni, J, nj, out):
        ii = np.ctypeslib.as_array(I, shape=(ni,))
        jj = np.ctypeslib.as_array(J, shape=(nj,))
        o = np.ctypeslib.as_array(out, shape=(2 * max(ni, nj),)).view(np.complex128)
        o[:] = A[ii[0], jj] if ni == 1 else A[ii, jj[0]]
    return ROWCOL_FN(gen)


def aca(A, tol):
    """aca.rs:23-179 on a matrix-backed generator (aca.rs:300-301)."""
    m, n = A.shape
    fn = _matrix_gen(A)
    U, V = _cbuf(m, min(m, n)), _cbuf(n, min(m, n))
    nrm = C.c_double()
    r = lib().oc_aca(m, n, tol, fn, None, _ptr(U), _ptr(V), C.byref(nrm))
    return U[:, :r].copy(), V[:, :r].copy(), nrm.value


class HMatrix:
    """h_matrix.rs:127-247 with a generic row/column generator."""

    def __init__(self, points, leaf, eta, tol, A=None, gen=None):
        self.points = np.ascontiguousarray(points, dtype=float)
        self._fn = _matrix_gen(A) if gen is None else ROWCOL_FN(gen)
        self.n = len(self.points)
        stride = self.points.shape[1]
        self.h = lib().oc_hmatrix_build(self.n, _ptr(self.points), stride, leaf, eta, tol, self._fn, None)
        if not self.h:
            raise ValueError("cluster tree construction failed")

    def __del__(self):
        try:
            lib().oc_hmatrix_free(self.h)
        except Exception:
            pass

    @property
    def norm(self):
        return lib().oc_hmatrix_norm(self.h)

    def gemv(self, alpha, x, beta, b):
        b = np.array(b, dtype=np.complex128)
        a = np.array([alpha.real, alpha.imag])
        be = np.array([beta.real, beta.imag])
        lib().oc_hmatrix_gemv(self.h, _ptr(a), _ptr(np.ascontiguousarray(x, dtype=np.complex128)), _ptr(be), _ptr(b))
        return b

    def to_full(self):
        A = _cbuf(self.n, self.n)
        lib().oc_hmatrix_to_full(self.h, _ptr(A), self.n)
        return A

    def stats(self):
        s = np.zeros(4, dtype=np.int64)
        lib().oc_hmatrix_stats(self.h, _ptr(s))
        return dict(admissible=int(s[0]), inadmissible=int(s[1]), stored=int(s[2]), rank_sum=int(s[3]))


def block_list(points, leaf, eta):
    pts = np.ascontiguousarray(points, dtype=float)
    bl = OcBlockList()
    if lib().oc_block_list(len(pts), _ptr(pts), pts.shape[1], leaf, eta, C.byref(bl)):
        raise ValueError("cluster tree construction failed")
    nb = bl.nblocks
    ro = np.ctypeslib.as_array(bl.row_off, shape=(nb + 1,)).copy()
    co = np.ctypeslib.as_array(bl.col_off, shape=(nb + 1,)).copy()
    rows = np.ctypeslib.as_array(bl.rows, shape=(max(ro[-1], 1),)).copy()[:ro[-1]]
    cols = np.ctypeslib.as_array(bl.cols, shape=(max(co[-1], 1),)).copy()[:co[-1]]
    adm = np.ctypeslib.as_array(bl.admissible, shape=(max(nb, 1),)).copy()[:nb]
    diam = bl.root_diameter
    lib().oc_blocklist_free(C.byref(bl))
    return dict(row_off=ro, rows=rows, col_off=co, cols=cols, admissible=adm, root_diameter=diam)


def block_tree_path_admissible(points, leaf, eta, path):
    pts = np.ascontiguousarray(points, dtype=float)
    p = np.ascontiguousarray(path, dtype=np.int32)
    return lib().oc_block_tree_path_admissible(len(pts), _ptr(pts), pts.shape[1], leaf, eta, _ptr(p), len(p))


# ---- postprocess.rs:15-67: the CSV writers ----------------------------------
def rust_f64_display(v):
    """Rust's `f64::to_string()` (core::fmt Display for f64): the shortest
    round-trip digits (Python's repr finds the same digits) laid out without an
    exponent, integral values without a decimal point, NaN / inf / -inf."""
    import decimal
    v = float(v)
    if v != v:
        return "NaN"
    if v in (float("inf"), float("-inf")):
        return "inf" if v > 0 else "-inf"
    d = decimal.Decimal(repr(v))
    sign, digits, exp = d.as_tuple()
    ds = "".join(map(str, digits)).lstrip("0") or "0"
    # value = ds * 10**exp with ds stripped of leading zeros; drop trailing zeros
    # of the digit string into the exponent
    stripped = ds.rstrip("0") or "0"
    exp += len(ds) - len(stripped)
    ds = stripped
    if ds == "0":
        body = "0"
    elif exp >= 0:
        body = ds + "0" * exp
    else:
        point = len(ds) + exp  # digits before the decimal point
        body = ("0." + "0" * (-point) + ds) if point <= 0 else ds[:point] + "." + ds[point:]
    return ("-" if sign else "") + body


def csv_results_at_frequency(field_points, scattered, incident, pressure=True):
    """The bytes of postprocess.rs:15-44 (csv 1.3.1 Writer: comma, "\\n")."""
    on = "pre" if pressure else "vpo"
    f = rust_f64_display
    lines = ["index,x,y,z,%s_re,%s_im,inc_re,inc_im" % (on, on)]
    for i, (p, s, c) in enumerate(zip(field_points, scattered, incident)):
        lines.append(",".join([str(i), f(p[0]), f(p[1]), f(p[2]), f(s.real), f(s.imag), f(c.real), f(c.imag)]))
    return ("\n".join(lines) + "\n").encode()


def csv_results_at_point(freqs, scattered, incident, index, pressure=True):
    """The bytes of postprocess.rs:47-67; scattered / incident: nfreq x nfp."""
    on = "pre" if pressure else "vpo"
    f = rust_f64_display
    lines = ["freq,%s_re,%s_im,inc_re,inc_im" % (on, on)]
    for fr, s, c in zip(freqs, scattered, incident):
        lines.append(",".join([f(fr), f(s[index].real), f(s[index].imag), f(c[index].real), f(c[index].imag)]))
    return ("\n".join(lines) + "\n").encode()
