"""C++ layer (include/pagani_gb300.cuh): Workspace<T, ndim>::integrate with user
functors, the reference's interface (cuda/pagani/quad/GPUquad/Workspace.cuh:23-70).

The CPU test compiles the header with nvcc (no GPU needed); the GPU test builds
tests/cpp/workspace_check.cu against the library and runs it: functors that
spell out a family's operations must give bit-identical results to the
library's families, per integral and per region.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "workspace_check.cu")
BUILD = os.path.join(ROOT, "tests", "cpp", "_build")


def _nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        pytest.skip("nvcc not available")
    return exe


def _flags():
    return ["-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-I" + os.path.join(ROOT, "include")]


def test_header_compiles():
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "workspace_check.o")
    subprocess.check_call([_nvcc()] + _flags() + ["-c", SRC, "-o", out])
    assert os.path.getsize(out) > 0


def test_functor_shapes_compile():
    """Functor shapes of the reference's callers (host-device, non-const, float
    arguments, integral return, device pointers, template operators) compile."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "functor_shapes.cu")
    out = os.path.join(BUILD, "functor_shapes.o")
    subprocess.check_call([_nvcc()] + _flags() + ["-c", src, "-o", out])
    assert os.path.getsize(out) > 0


@pytest.mark.parametrize("reference_first", [0, 1])
def test_header_with_reference_types_either_order(reference_first):
    """numint::integration_result and quad::Volume come from whichever header is
    included first (the reference's integrand-side headers include them)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "interop_check.cu")
    out = os.path.join(BUILD, f"interop_{reference_first}.o")
    subprocess.check_call([_nvcc()] + _flags() + [f"-DREFERENCE_FIRST={reference_first}", "-c", src, "-o", out])
    assert os.path.getsize(out) > 0


@pytest.mark.gpu
def test_workspace_functors_match_families(lib):
    from gpuintegration_gb300 import _build
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "workspace_check")
    libdir = os.path.dirname(_build.LIB)
    subprocess.check_call([_nvcc()] + _flags() + ["-cudart", "shared", SRC, "-L" + libdir, "-lpagani_gb300",
                                                  "-Xlinker", "-rpath," + libdir, "-o", exe])
    p = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(p.stdout)
    lines = p.stdout.strip().splitlines()
    assert p.returncode == 0, p.stdout + p.stderr
    assert lines and lines[-1].startswith("DONE 0 failures")
    names = {ln.split()[1] for ln in lines if ln.startswith("PASS")}
    for case in ("gauss3_unit", "gauss5_box", "gauss8_unit", "gauss10_unit", "peak6_box_norelerr", "xy_unit",
                 "xy_value", "nan3", "tabulated3", "regions5", "subregions5x5_peak2", "predict_split_peak2",
                 "predict_split_snapshot", "mcubes_gauss3", "quad_mcubes_gauss3", "mcubes_value"):
        assert case in names, case


@pytest.mark.gpu
def test_integer_pipe_multiply_matches_fp64_multiply():
    """pg::mul_rn_int, the evaluation kernel's double multiply on the integer
    pipe, equals __dmul_rn bit for bit on 2^30 products (random patterns,
    exact products and ties, the whole exponent range with zeros and infinities)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "mul_check.cu")
    exe = os.path.join(BUILD, "mul_check")
    subprocess.check_call([_nvcc(), "-std=c++17", "-O3", "--fmad=false", "-gencode", "arch=compute_103a,code=sm_103a",
                           src, "-o", exe])
    p = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(p.stdout)
    assert p.returncode == 0 and p.stdout.startswith("PASS"), p.stdout + p.stderr


def _reference_tree():
    ref = os.environ.get("REF") or os.path.join(ROOT, "..", "reference")
    return ref if os.path.isfile(os.path.join(ref, "common", "cuda", "Interp1D.cuh")) else None


@pytest.mark.parametrize("helpers_first", [0, 1])
def test_reference_helpers_compile_in_functors(helpers_first):
    """Functors built on the reference's Interp1D/2D/3D, polynomial and
    cudaDynamicArray (test/cuda/common/StatefulIntegrand.cu:34-97) compile
    against the C++ layer, with this library's helpers header included before
    or after the reference's.  Needs the reference tree (REF); skipped without it."""
    ref = _reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "ref_helpers_check.cu")
    out = os.path.join(BUILD, f"ref_helpers_check_{helpers_first}.o")
    subprocess.check_call([_nvcc()] + _flags() + ["-I" + ref, "-I" + os.path.join(ref, "externals"),
                                                  f"-DHELPERS_FIRST={helpers_first}", "-c", src, "-o", out])
    assert os.path.getsize(out) > 0


def test_helpers_error_behaviour():
    """Bad tables throw std::invalid_argument before allocating; without a CUDA
    device the helpers' allocations throw std::bad_alloc; empty tables give NaN
    (tests/cpp/helpers_errors.cu, run on the host)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "helpers_errors.cu")
    exe = os.path.join(BUILD, "helpers_errors")
    subprocess.check_call([_nvcc()] + _flags() + [src, "-o", exe])
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(p.stdout)
    lines = p.stdout.strip().splitlines()
    assert p.returncode == 0, p.stdout + p.stderr
    assert lines and lines[-1].startswith("DONE 0 failures")


def test_helpers_header_compiles():
    """include/pagani_gb300_helpers.cuh with the C++ layer: the GPU check program compiles (no GPU needed)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "helpers_check.cu")
    out = os.path.join(BUILD, "helpers_check.o")
    subprocess.check_call([_nvcc()] + _flags() + ["-c", src, "-o", out])
    assert os.path.getsize(out) > 0


@pytest.mark.gpu
def test_stateful_helper_functors_run(lib):
    """The library's integrand-side helpers (include/pagani_gb300_helpers.cuh):
    the reference's known answers for Interp1D/2D/3D, cudaDynamicArray and
    stateful integrands; device equals host bit for bit and agrees with the
    reference's interpolation formulas to 1e-14; functors holding them through
    Workspace::integrate against exact integrals; table copies share one
    device store."""
    from gpuintegration_gb300 import _build
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "helpers_check.cu")
    exe = os.path.join(BUILD, "helpers_check")
    libdir = os.path.dirname(_build.LIB)
    subprocess.check_call([_nvcc()] + _flags() + ["-cudart", "shared", src, "-L" + libdir, "-lpagani_gb300",
                                                  "-Xlinker", "-rpath," + libdir, "-o", exe])
    p = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(p.stdout)
    lines = p.stdout.strip().splitlines()
    assert p.returncode == 0, p.stdout + p.stderr
    assert lines and lines[-1].startswith("DONE 0 failures")
    names = {ln.split()[1] for ln in lines if ln.startswith("PASS")}
    for case in ("ref_interp1d_exact_at_knots", "ref_interp1d_quadratic", "ref_interp2d_value", "ref_interp2d_clamp",
                 "ref_interp2d_exact_at_knots", "ref_interp2d_bilinear", "ref_interp3d_linear",
                 "ref_interp3d_quadratic", "ref_interp3d_clamp", "ref_dynamic_array", "dynamic_array_device_copy",
                 "ref_stateful_array", "ref_stateful_dynamic_array", "interp1d_device_equals_host",
                 "interp1d_vs_reference_formula", "interp2d_device_equals_host", "interp2d_vs_reference_formula",
                 "interp3d_device_equals_host", "interp3d_vs_reference_formula", "polynomial_device_equals_host",
                 "polynomial_vs_horner", "interp_stream_input", "interp_rejects_unordered_axis", "interp1d_3",
                 "interp2d_4", "interp3d_3", "polynomial_dynamic_array_2", "interp_copies_share_device_store"):
        assert case in names, case
