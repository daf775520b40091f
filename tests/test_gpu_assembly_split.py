"""The refined form's split assembly (assemble_ff_kernel in
csrc/assembly32.cu): every entry of A_f = alpha_f H_f + beta_f G_f
(influence_matrix.rs:64-98 with the factors of :130-162) evaluated in
float-float on the FP32 pipe and stored as its FP32 rounding plus the FP32
rounding of the remainder.  Summed in FP64 it must agree with the FP64 oracle
at FP64 level (5e-14 of the largest entry), far below the FP32 operator of
the mixed form (~6e-8): for classical and Burton-Miller operators, triangles and quads, the
rigid, pressure and impedance conditions, evenly spaced wavenumbers (e^{ik r}
by recurrence) and a list that is not (sine and cosine per frequency), and
k r up to 40 (argument reduction)."""
import numpy as np
import pytest

from conftest import sphere_input
from oracle import oracle as O

pytestmark = pytest.mark.gpu
bem = pytest.importorskip("cc_abstemious_gb300")
from cc_abstemious_gb300 import workloads  # noqa: E402

# measured on a GB300: max 1e-15 .. 1.7e-14, Frobenius 6e-16 .. 7e-15 (the
# FP64 oracle's own rounding is of the same order)
SPLIT_MAX = 5e-14   # max |A - A64| / max |A64|
SPLIT_FRO = 2e-14   # ||A - A64||_F / ||A64||_F


@pytest.fixture(scope="module")
def ctx():
    return bem.Context.default()


def _check(ctx, inp):
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    op = O.Problem(inp)
    nf = len(pd.frequencies)
    A = bem.assemble_operator(pd, "split")
    A32 = bem.assemble_operator(pd, "fp32")
    worst = []
    for f in range(nf):
        op.set_frequency_index(f)
        H, G = op.dense_surface(nthreads=8)
        a, b = op.lhs_factors()
        ref = a * H + b * G
        emax = np.max(np.abs(A[f] - ref)) / np.max(np.abs(ref))
        efro = np.linalg.norm(A[f] - ref) / np.linalg.norm(ref)
        e32 = np.linalg.norm(A32[f] - ref) / np.linalg.norm(ref)
        worst.append((emax, efro, e32))
        assert emax < SPLIT_MAX and efro < SPLIT_FRO, (f, emax, efro)
        assert efro < 1e-4 * e32, (f, efro, e32)
    print("split max/fro, fp32 fro:", ["%.2e %.2e %.2e" % w for w in worst])


def test_rounded_operator_is_the_fp32_rounding(ctx, tmp_path):
    """The mixed_rounded form's operator (the split assembly's first plane) is
    the FP32 rounding of the FP64 entry: equal to numpy's rounding of the
    oracle's FP64 operator except where the float-float value and the oracle
    fall on opposite sides of a rounding boundary (then one FP32 ulp)."""
    inp = workloads.perturbed_sphere_input(str(tmp_path), 23, 700, [1.0, 4.0, 7.0])
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    op = O.Problem(inp)
    R = bem.assemble_operator(pd, "rounded")
    for f in range(len(pd.frequencies)):
        op.set_frequency_index(f)
        H, G = op.dense_surface(nthreads=8)
        a, b = op.lhs_factors()
        ref = (a * H + b * G).astype(np.complex64)
        got = R[f].astype(np.complex64)
        same = np.mean((got.real == ref.real) & (got.imag == ref.imag))
        assert same > 0.9999, same
        ulp = np.spacing(np.maximum(np.abs(ref.real), np.abs(ref.imag)).astype(np.float32))
        assert np.all(np.abs(got.real - ref.real) <= ulp) and np.all(np.abs(got.imag - ref.imag) <= ulp)


@pytest.mark.parametrize("kw", [{}, {"method_type": "BurtonMiller"},
                                {"surface_bc": {"bc_type": "Pressure", "value": [0.0, 0.0]}},
                                {"method_type": "BurtonMiller", "surface_bc": {"bc_type": "Pressure",
                                                                               "value": [0.3, -0.1]}}])
def test_sphere_evenly_spaced(ctx, kw):
    _check(ctx, sphere_input(frequency={"List": {"values": [100.0, 300.0, 500.0, 700.0]}}, **kw))


def test_quads_uneven_list_high_kr(ctx):
    inp = sphere_input("sphere_quad.vtk", body_index=2, method_type="BurtonMiller",
                       frequency={"List": {"values": [120.0, 2000.0, 9549.0]}})
    _check(ctx, inp)


def test_impedance_body(ctx, tmp_path):
    inp = workloads.perturbed_sphere_input(str(tmp_path), 21, 900, [0.5, 2.0, 3.5, 5.0, 6.5, 8.0])
    _check(ctx, inp)
