"""GB300 (sm_103a) implementation of the cc_abstemious BEM hot path.

The Python layer mirrors the reference's module API (src/influence_matrix.rs,
src/incident_wave.rs, src/solve.rs, src/postprocess.rs, src/analysis.rs) over
the C ABI of libbem_gb300.so (include/bem.h).  All numerical work runs in the
library's CUDA kernels; this module only marshals arguments.

    from cc_abstemious_gb300 import Analysis
    a = Analysis()
    a.input_from_file("input.json")
    a.run()
    a.write_results_at_frequency(0)
"""
import ctypes as C
import json
import os

import numpy as np

from . import _lib
from ._lib import (BemError, FORM_MIXED, FORM_MIXED_ROUNDED, FORM_PLAIN_FP64, FORM_REFINED, MEM_DEVICE, MEM_HOST,
                   PRECOND_BLOCK_JACOBI, PRECOND_LEARNED, PRECOND_LU, PRECOND_NONE, SIDE_LHS, SIDE_RHS, SolveReport)

__all__ = ["Analysis", "Context", "PreData", "FPResult", "BemError", "get_dense_surface_matrices",
           "get_dense_field_matrices", "get_surface_row_or_column", "get_incident_surface", "get_incident_field",
           "solve_for_surface", "solve_lu", "gmres", "get_field", "evaluate_field", "convert_results",
           "write_results_at_frequency", "write_results_at_point", "EqnSide", "HMatrix"]


class EqnSide:
    """influence_matrix.rs:164-167"""
    RHS = SIDE_RHS
    LHS = SIDE_LHS


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _dptr(t):
    return C.c_void_p(t.data_ptr())


class Context:
    """One CUDA device and stream (bem_ctx)."""

    _default = {}

    def __init__(self, device=0):
        self.lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self.lib.bem_ctx_create(device, C.byref(h)))
        self.h = h
        self.device = device

    @classmethod
    def default(cls, device=0):
        if device not in cls._default:
            cls._default[device] = Context(device)
        return cls._default[device]

    def check(self, status):
        _lib.check(status, self.h)

    @property
    def kernel_launches(self):
        return self.lib.bem_ctx_kernel_launches(self.h)

    @property
    def stream(self):
        """Raw cudaStream_t of the context (for torch.cuda.ExternalStream)."""
        return self.lib.bem_ctx_stream(self.h)

    def set_profiling(self, on):
        self.check(self.lib.bem_ctx_set_profiling(self.h, 1 if on else 0))

    def profile(self):
        out = {}
        buf = C.create_string_buffer(128)
        for i in range(self.lib.bem_ctx_profile_count(self.h)):
            ms, launches, nbytes = C.c_double(), C.c_int64(), C.c_double()
            self.check(self.lib.bem_ctx_profile_get(self.h, i, buf, 128, C.byref(ms), C.byref(launches),
                                                    C.byref(nbytes)))
            out[buf.value.decode()] = {"ms": ms.value, "launches": launches.value, "bytes": nbytes.value}
        return out

    def __del__(self):
        try:
            if self.h:
                self.lib.bem_ctx_destroy(self.h)
                self.h = None
        except Exception:
            pass


class PreData:
    """UserInput + PreData (input_data.rs:80-92, preprocess.rs:24-124): the
    parsed JSON, the mesh and its collocation points computed on the device."""

    def __init__(self, handle, ctx):
        self.h = handle
        self.ctx = ctx
        info = _lib.ProblemInfo()
        ctx.check(ctx.lib.bem_problem_get_info(self.h, C.byref(info)))
        self._info = info
        self.n = int(info.num_eqn)
        self.nfp = int(info.num_field_points)
        self.frequencies = np.zeros(int(info.num_frequencies))
        ctx.check(ctx.lib.bem_problem_frequencies(self.h, _ptr(self.frequencies)))
        self.ifreq = 0

    @classmethod
    def from_json(cls, text, base_dir=None, ctx=None):
        ctx = ctx or Context.default()
        h = C.c_void_p()
        ctx.check(ctx.lib.bem_problem_from_json(ctx.h, text.encode(), base_dir.encode() if base_dir else None,
                                                C.byref(h)))
        pd = cls(h, ctx)
        pd.field_points = np.array(json.loads(text)["output"]["field_points"], dtype=float).reshape(-1, 3)
        return pd

    @classmethod
    def from_dict(cls, d, base_dir=None, ctx=None):
        return cls.from_json(json.dumps(d), base_dir, ctx)

    @classmethod
    def from_file(cls, path, ctx=None):
        ctx = ctx or Context.default()
        h = C.c_void_p()
        ctx.check(ctx.lib.bem_problem_from_file(ctx.h, os.fsencode(path), C.byref(h)))
        pd = cls(h, ctx)
        with open(path) as f:
            pd.field_points = np.array(json.load(f)["output"]["field_points"], dtype=float).reshape(-1, 3)
        return pd

    @property
    def info(self):
        i = self._info
        d = {k: getattr(i, k) for k, _ in i._fields_}
        for k in ("incident_vec", "incident_amp", "bc_value"):
            d[k] = list(d[k])
        return d

    def set_frequency_index(self, i):
        self.ctx.check(self.ctx.lib.bem_problem_set_frequency_index(self.h, i))
        self.ifreq = i

    def get_frequency(self):
        return float(self.frequencies[self.ifreq])

    def get_cpts(self):
        out = np.zeros((self.n, 8))
        self.ctx.check(self.ctx.lib.bem_collocation(self.ctx.h, self.h, _ptr(out)))
        return out

    def __del__(self):
        try:
            if self.h:
                self.ctx.lib.bem_problem_destroy(self.h)
                self.h = None
        except Exception:
            pass


def _c(n, m=None):
    return np.zeros((n,) if m is None else (n, m), dtype=np.complex128, order="F")


# ---- influence_matrix.rs ---------------------------------------------------
def get_dense_surface_matrices(pd, out=None):
    """influence_matrix.rs:64-98.  Returns (H, G) as n x n complex128
    (column-major numpy arrays), or fills `out=(H, G)` torch CUDA tensors."""
    ctx = pd.ctx
    if out is not None:
        H, G = out
        ld = H.stride(1)
        ctx.check(ctx.lib.bem_get_dense_surface_matrices(ctx.h, pd.h, _dptr(H), _dptr(G), ld, MEM_DEVICE))
        return H, G
    H, G = _c(pd.n, pd.n), _c(pd.n, pd.n)
    ctx.check(ctx.lib.bem_get_dense_surface_matrices(ctx.h, pd.h, _ptr(H), _ptr(G), pd.n, MEM_HOST))
    return H, G


def get_system_matrix_fp32(pd):
    """The mixed form's single-precision alpha H + beta G at the current
    frequency (n x n complex64, column-major)."""
    A = np.zeros((pd.n, pd.n), dtype=np.complex64, order="F")
    pd.ctx.check(pd.ctx.lib.bem_get_system_matrix_fp32(pd.ctx.h, pd.h, _ptr(A), pd.n))
    return A


def get_dense_field_matrices(pd):
    """influence_matrix.rs:101-127.  Returns (M, L), nfp x n."""
    ctx = pd.ctx
    M, L = _c(pd.nfp, pd.n), _c(pd.nfp, pd.n)
    if pd.nfp:
        ctx.check(ctx.lib.bem_get_dense_field_matrices(ctx.h, pd.h, _ptr(M), _ptr(L), pd.nfp, MEM_HOST))
    return M, L


def get_surface_row_or_column(pd, i, j, side):
    """influence_matrix.rs:170-193: i or j must be a singleton."""
    ctx = pd.ctx
    I = np.ascontiguousarray(np.atleast_1d(i), dtype=np.int64)
    J = np.ascontiguousarray(np.atleast_1d(j), dtype=np.int64)
    out = _c(max(len(I), len(J)))
    ctx.check(ctx.lib.bem_get_surface_row_or_column(ctx.h, pd.h, _ptr(I), len(I), _ptr(J), len(J), side, _ptr(out)))
    return out


# ---- incident_wave.rs --------------------------------------------------------
def get_incident_surface(pd):
    """incident_wave.rs:7-63"""
    out = _c(pd.n)
    pd.ctx.check(pd.ctx.lib.bem_get_incident_surface(pd.ctx.h, pd.h, _ptr(out)))
    return out


def get_incident_field(pd):
    """incident_wave.rs:66-99"""
    out = _c(pd.nfp)
    if pd.nfp:
        pd.ctx.check(pd.ctx.lib.bem_get_incident_field(pd.ctx.h, pd.h, _ptr(out)))
    return out


# ---- solve.rs ----------------------------------------------------------------
def solve_for_surface(pd, rhs_inc):
    """solve.rs:11-22 (plain FP64 form).  Returns (phi, vn, report)."""
    rhs = np.ascontiguousarray(rhs_inc, dtype=np.complex128)
    phi, vn = _c(pd.n), _c(pd.n)
    rep = SolveReport()
    st = pd.ctx.lib.bem_solve_for_surface(pd.ctx.h, pd.h, _ptr(rhs), _ptr(phi), _ptr(vn), C.byref(rep))
    if st not in (0, 3):
        pd.ctx.check(st)
    return phi, vn, rep.as_dict()


def solve_lu(A, b, ctx=None):
    """solve.rs:166-171: returns A^-1 b (FP64 partial-pivot LU on the device)."""
    ctx = ctx or Context.default()
    A = np.asfortranarray(A, dtype=np.complex128)
    x = np.array(b, dtype=np.complex128)
    ctx.check(ctx.lib.bem_solve_lu(ctx.h, A.shape[0], _ptr(A), A.shape[0], _ptr(x), MEM_HOST))
    return x


def gmres(A, b, max_it, tol, ctx=None):
    """gmres.rs:35-59 GMRES::solve with a dense matrix.  Returns (x, report)."""
    ctx = ctx or Context.default()
    A = np.asfortranarray(A, dtype=np.complex128)
    x = np.array(b, dtype=np.complex128)
    rep = SolveReport()
    st = ctx.lib.bem_gmres_solve(ctx.h, A.shape[0], _ptr(A), A.shape[0], max_it, tol, _ptr(x), C.byref(rep),
                                 MEM_HOST)
    if st not in (0, 3):
        ctx.check(st)
    return x, rep.as_dict()


def get_field(pd, M, L, phi, vn, phi_inc_fp):
    """solve.rs:173-185"""
    out = _c(pd.nfp)
    if not pd.nfp:
        return out
    M = np.asfortranarray(M, dtype=np.complex128)
    L = np.asfortranarray(L, dtype=np.complex128)
    args = [np.ascontiguousarray(v, dtype=np.complex128) for v in (phi, vn, phi_inc_fp)]
    pd.ctx.check(pd.ctx.lib.bem_get_field(pd.ctx.h, pd.h, _ptr(M), _ptr(L), pd.nfp, *[_ptr(a) for a in args],
                                          _ptr(out), MEM_HOST))
    return out


def evaluate_field(pd, phi, vn, phi_inc_fp=None):
    """Field without storing M and L (same result as get_field)."""
    out = _c(pd.nfp)
    if not pd.nfp:
        return out
    args = [np.ascontiguousarray(v, dtype=np.complex128) for v in (phi, vn)]
    inc = np.ascontiguousarray(phi_inc_fp, dtype=np.complex128) if phi_inc_fp is not None else None
    pd.ctx.check(pd.ctx.lib.bem_evaluate_field(pd.ctx.h, pd.h, _ptr(args[0]), _ptr(args[1]), _ptr(inc), _ptr(out)))
    return out


# ---- postprocess.rs ------------------------------------------------------------
class FPResult:
    """postprocess.rs:7-12"""

    def __init__(self, frequency, scattered, incident, radiated_power=0.0):
        self.frequency = frequency
        self.scattered = scattered
        self.incident = incident
        self.radiated_power = radiated_power


def convert_results(pd, results):
    """postprocess.rs:70-79: phi -> p = i omega rho phi when the output field is Pressure."""
    if not pd.info["output_pressure"]:
        return
    for r in results:
        for v in (r.scattered, r.incident):
            pd.ctx.check(pd.ctx.lib.bem_convert_to_pressure(pd.h, r.frequency, _ptr(v), len(v)))


def write_results_at_frequency(pd, result, path=None):
    """postprocess.rs:15-44 through bem_write_results_at_frequency (path None:
    the input's output.file)."""
    sc = np.ascontiguousarray(result.scattered, dtype=np.complex128)
    inc = np.ascontiguousarray(result.incident, dtype=np.complex128)
    pd.ctx.check(pd.ctx.lib.bem_write_results_at_frequency(pd.ctx.h, pd.h, path.encode() if path else None,
                                                           _ptr(sc), _ptr(inc)))


def write_results_at_point(pd, results, index, path=None):
    """postprocess.rs:47-67 through bem_write_results_at_point."""
    sc = np.ascontiguousarray(np.stack([r.scattered for r in results]), dtype=np.complex128)
    inc = np.ascontiguousarray(np.stack([r.incident for r in results]), dtype=np.complex128)
    pd.ctx.check(pd.ctx.lib.bem_write_results_at_point(pd.ctx.h, pd.h, path.encode() if path else None, index,
                                                       _ptr(sc), _ptr(inc)))


def format_f64(v):
    """Rust's f64 Display as the CSV writers print numbers (bem_format_f64)."""
    buf = C.create_string_buffer(512)
    n = _lib.load().bem_format_f64(float(v), buf, len(buf))
    if n < 0:
        raise BemError(6, "formatting failed")
    return buf.value.decode()


# ---- analysis.rs -----------------------------------------------------------------
class Analysis:
    """analysis.rs:22-128.  `run(form=...)` selects the plain FP64 drop-in
    form (default) or the batched mixed-precision form."""

    def __init__(self, ctx=None):
        self.ctx = ctx
        self._input = None
        self._base_dir = None
        self.predata = None
        self.results = []
        self.reports = []

    def input_from_file(self, path):
        with open(path) as f:
            self._input = f.read()
        self._base_dir = None  # the reference resolves mesh_file against the working directory

    def input_from_string(self, text):
        self._input = text

    def set_input(self, d, base_dir=None):
        self._input = json.dumps(d)
        self._base_dir = base_dir

    def run(self, form="plain", precond=None, check_vs_lu=False):
        if self._input is None:
            raise RuntimeError("No input found")
        ctx = self.ctx or Context.default()
        pd = PreData.from_json(self._input, self._base_dir, ctx)
        self.predata = pd
        nf, nfp = len(pd.frequencies), pd.nfp
        R = int(pd.info["num_rhs"])  # incident_wave + additional_incident_waves
        sc = np.zeros((R * nf, max(nfp, 1)), dtype=np.complex128)
        inc = np.zeros((R * nf, max(nfp, 1)), dtype=np.complex128)
        reps = (SolveReport * max(R * nf, 1))()
        f = {"plain": FORM_PLAIN_FP64, "mixed": FORM_MIXED, "refined": FORM_REFINED,
             "mixed_rounded": FORM_MIXED_ROUNDED}[form]
        pc = {None: PRECOND_NONE, "none": PRECOND_NONE, "block_jacobi": PRECOND_BLOCK_JACOBI,
              "learned": PRECOND_LEARNED, "lu": PRECOND_LU}[precond]
        st = ctx.lib.bem_run(ctx.h, pd.h, f, pc, _ptr(sc), _ptr(inc), reps, 1 if check_vs_lu else 0)
        ctx.check(st)
        # per incident wave (wave-major); results / reports are those of the
        # first wave, as the reference's single incident_wave
        self.results_by_rhs = [[FPResult(float(pd.frequencies[i]), sc[r * nf + i, :nfp].copy(),
                                         inc[r * nf + i, :nfp].copy()) for i in range(nf)] for r in range(R)]
        self.reports_by_rhs = [[reps[r * nf + i].as_dict() for i in range(nf)] for r in range(R)]
        self.results = self.results_by_rhs[0]
        self.reports = self.reports_by_rhs[0]

    def get_result(self):
        return self.results

    def surface_solution(self):
        pd = self.predata
        nf = len(pd.frequencies) * int(pd.info["num_rhs"])
        phi = np.zeros((nf, pd.n), dtype=np.complex128)
        vn = np.zeros((nf, pd.n), dtype=np.complex128)
        self.ctx_or_default().check(pd.ctx.lib.bem_last_surface(pd.ctx.h, pd.h, _ptr(phi), _ptr(vn)))
        return phi, vn

    def ctx_or_default(self):
        return self.ctx or Context.default()

    def write_results_at_frequency(self, ifreq, path=None):
        """analysis.rs:121-123"""
        write_results_at_frequency(self.predata, self.results[ifreq], path)

    def write_results_at_point(self, index, path=None):
        """analysis.rs:124-126"""
        write_results_at_point(self.predata, self.results, index, path)


_PRECONDS = {None: PRECOND_NONE, "none": PRECOND_NONE, "block_jacobi": PRECOND_BLOCK_JACOBI,
             "learned": PRECOND_LEARNED, "lu": PRECOND_LU}


def run_batch(predatas, precond=None, check_vs_lu=False, max_operator_bytes=0, ctx=None):
    """Several bodies in one batch (mixed form, no reference counterpart: the
    reference runs one Analysis per body).  Returns, per body, a list of
    FPResult (pressure / potential as Analysis.run leaves them) and the
    per-frequency solve reports."""
    ctx = ctx or (predatas[0].ctx if predatas else Context.default())
    nb = len(predatas)
    outs, ptrs_s, ptrs_i, reps = [], (C.c_void_p * max(nb, 1))(), (C.c_void_p * max(nb, 1))(), []
    rep_ptrs = (C.c_void_p * max(nb, 1))()
    handles = (C.c_void_p * max(nb, 1))()
    for b, pd in enumerate(predatas):
        nf, nfp = len(pd.frequencies), pd.nfp
        sc = np.zeros((nf, max(nfp, 1)), dtype=np.complex128)
        inc = np.zeros((nf, max(nfp, 1)), dtype=np.complex128)
        r = (SolveReport * max(nf, 1))()
        outs.append((sc, inc))
        reps.append(r)
        ptrs_s[b], ptrs_i[b] = sc.ctypes.data, inc.ctypes.data
        rep_ptrs[b] = C.cast(r, C.c_void_p)
        handles[b] = pd.h
    ctx.check(ctx.lib.bem_run_batch(ctx.h, handles, nb, _PRECONDS[precond], ptrs_s, ptrs_i, rep_ptrs,
                                    1 if check_vs_lu else 0, int(max_operator_bytes)))
    results = []
    for b, pd in enumerate(predatas):
        nf, nfp = len(pd.frequencies), pd.nfp
        sc, inc = outs[b]
        results.append(([FPResult(float(pd.frequencies[i]), sc[i, :nfp].copy(), inc[i, :nfp].copy())
                         for i in range(nf)], [reps[b][i].as_dict() for i in range(nf)]))
    return results


def assemble_operator(pd, kind="split", f0=0, nf=None):
    """The operators A_f = alpha_f H_f + beta_f G_f of frequencies f0 ..
    f0 + nf - 1 of a problem as the batched forms assemble them: kind "fp32"
    (the mixed form), "split" (the refined form: FP32 rounding plus FP32
    remainder, returned summed in FP64) or "rounded" (the mixed_rounded form:
    that FP32 rounding alone).  Returns an (nf, n, n) array."""
    nf = len(pd.frequencies) - f0 if nf is None else nf
    n = pd.n
    A = np.zeros((nf, n, n), dtype=np.complex128)  # each [f] holds A_f^T (column-major fill)
    k = {"fp32": 0, "split": 1, "rounded": 2}[kind]
    pd.ctx.check(pd.ctx.lib.bem_assemble_operator(pd.ctx.h, pd.h, k, f0, nf, _ptr(A), n))
    return np.ascontiguousarray(np.transpose(A, (0, 2, 1)))


def cluster_tree(point_sets, leaf, eta=None, ctx=None):
    """Cluster trees (cluster.rs:35-105) of one or several point sets and,
    with eta, their block trees (block.rs:38-93), built on the device in one
    pass.  point_sets: an (n, >= 3) array or a list of them.  Per set returns
    dict(perm, leaves [(begin, end)], blocks [(row begin, row end, column
    begin, column end, admissible)], root_diameter); a cluster's points are
    perm[begin:end], and leaves and blocks are in the reference's depth-first
    order."""
    ctx = ctx or Context.default()
    single = isinstance(point_sets, np.ndarray)
    sets = [np.ascontiguousarray(point_sets if single else p, dtype=np.float64) for p in
            ([point_sets] if single else point_sets)]
    stride = sets[0].shape[1]
    if any(p.ndim != 2 or p.shape[1] != stride or stride < 3 for p in sets):
        raise ValueError("point sets must be (n, k) arrays with one k >= 3")
    npts = np.array([len(p) for p in sets], dtype=np.int64)
    pts = np.concatenate(sets) if npts.sum() else np.zeros((1, stride))
    perm = np.zeros(max(int(npts.sum()), 1), dtype=np.int64)
    diam = np.zeros(len(sets))
    nl, nb = C.c_int64(), C.c_int64()
    e = -1.0 if eta is None else float(eta)
    lcap, bcap = max(int(npts.sum()), 1), 4 * max(int(npts.sum()), 1)
    while True:
        leaves = np.zeros((lcap, 3), dtype=np.int64)
        blocks = np.zeros((bcap, 6), dtype=np.int64)
        st = ctx.lib.bem_cluster_tree(ctx.h, len(sets), _ptr(npts), _ptr(pts), stride, int(leaf), e, _ptr(perm),
                                      _ptr(leaves), lcap, C.byref(nl), _ptr(blocks), bcap, C.byref(nb), _ptr(diam))
        if st != 0 and (nl.value > lcap or nb.value > bcap):
            lcap, bcap = max(lcap, nl.value), max(bcap, nb.value)
            continue
        ctx.check(st)
        break
    leaves, blocks = leaves[:nl.value], blocks[:nb.value]
    out, p0 = [], 0
    for s, n in enumerate(npts):
        lv = leaves[leaves[:, 0] == s][:, 1:]
        bk = blocks[blocks[:, 0] == s][:, 1:]
        out.append(dict(perm=perm[p0:p0 + n].copy(), leaves=lv, blocks=bk, root_diameter=float(diam[s])))
        p0 += n
    return out[0] if single else out


class HMatrix:
    """h_matrix.rs:110-247 over a problem's collocation points."""

    def __init__(self, pd, side=SIDE_LHS):
        self.pd = pd
        h = C.c_void_p()
        pd.ctx.check(pd.ctx.lib.bem_hmatrix_build(pd.ctx.h, pd.h, side, C.byref(h)))
        self.h = h
        self.n = pd.n

    @property
    def norm(self):
        return self.pd.ctx.lib.bem_hmatrix_norm(self.h)

    def stats(self):
        s = np.zeros(4, dtype=np.int64)
        self.pd.ctx.check(self.pd.ctx.lib.bem_hmatrix_stats(self.h, _ptr(s)))
        return dict(admissible=int(s[0]), inadmissible=int(s[1]), stored=int(s[2]), rank_sum=int(s[3]))

    def gemv(self, alpha, x, beta, b):
        b = np.array(b, dtype=np.complex128)
        x = np.ascontiguousarray(x, dtype=np.complex128)
        a = _lib.Cplx(alpha.real, alpha.imag)
        be = _lib.Cplx(beta.real, beta.imag)
        self.pd.ctx.check(self.pd.ctx.lib.bem_hmatrix_gemv(self.pd.ctx.h, self.h, a, _ptr(x), be, _ptr(b)))
        return b

    def to_full(self):
        A = _c(self.n, self.n)
        self.pd.ctx.check(self.pd.ctx.lib.bem_hmatrix_to_full(self.pd.ctx.h, self.h, _ptr(A), self.n))
        return A

    def __del__(self):
        try:
            if self.h:
                self.pd.ctx.lib.bem_hmatrix_destroy(self.h)
                self.h = None
        except Exception:
            pass


# ---- learned preconditioner ------------------------------------------------------
def learned_num_params():
    return int(_lib.load().bem_learned_num_params())


def learned_train(problems, steps=200, nprobe=8, lr=1e-3, seed=0, ctx=None):
    """Train the context's preconditioner network on the operators of
    `problems` (PreData, all their frequencies).  Returns the per-step losses
    E ||A M z - z||^2 / ||z||^2 relative to block-Jacobi's on the same system
    (1: no better than block-Jacobi)."""
    ctx = ctx or problems[0].ctx
    arr = (C.c_void_p * len(problems))(*[p.h for p in problems])
    losses = np.zeros(max(steps, 1))
    ctx.check(ctx.lib.bem_learned_train(ctx.h, arr, len(problems), steps, nprobe, lr, seed, _ptr(losses)))
    return losses[:steps]


def learned_get_weights(ctx=None):
    ctx = ctx or Context.default()
    w = np.zeros(learned_num_params(), dtype=np.float32)
    ctx.check(ctx.lib.bem_learned_get_weights(ctx.h, _ptr(w)))
    return w


def learned_set_weights(w, ctx=None):
    ctx = ctx or Context.default()
    w = np.ascontiguousarray(w, dtype=np.float32)
    ctx.check(ctx.lib.bem_learned_set_weights(ctx.h, _ptr(w)))


def learned_mlp_eval(features, dO=None, ctx=None):
    """Network outputs (P x 2) for P x 16 features and, with dO, the gradient of
    sum(dO * outputs) with respect to the parameters."""
    ctx = ctx or Context.default()
    F = np.ascontiguousarray(features, dtype=np.float32)
    P = F.shape[0]
    out = np.zeros((P, 2), dtype=np.float32)
    grad = None
    if dO is not None:
        dO = np.ascontiguousarray(dO, dtype=np.float32)
        grad = np.zeros(learned_num_params(), dtype=np.float32)
    ctx.check(ctx.lib.bem_learned_mlp_eval(ctx.h, P, _ptr(F), _ptr(dO), _ptr(out), _ptr(grad)))
    return (out, grad) if dO is not None else out
