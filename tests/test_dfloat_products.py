"""Accuracy of the double-float 3x3 products (su3.cuh), measured on the host:
the product functions are host-and-device code, so a host build of the same
source checks the arithmetic without a GPU. Random complex Gaussian matrices
at scales 1e-3..1e3, 40,000 products of each kind, against long double;
errors relative to |row i of A| |column j of B| (+ |C_ij|).

Measured here: the fixed-grid product (dfg_matmul) rms 1.2e-13 (2^-43.0),
max 3.6e-12 (2^-38.0), accumulating 1.3e-13 / 2.7e-12; the TwoSum form
(df_matmul) rms 2.7e-15 (2^-48.4), max 3.4e-14 (2^-44.8); a raw grid pair as
the next operand rms 1.7e-13. The grid product's tail is its fp32 correction
word: up to twelve rounding residuals of half a grid step (2^-21 of the bound)
each, plus the cross terms, summed in fp32 (2^-24 of the word per addition).
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "native", "dfloat_products.cu")
INC = os.path.join(ROOT, "gaugefields.jl_gb300", "csrc")


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


@pytest.fixture(scope="module")
def measured(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("dfp") / "dfloat_products")
    try:
        r = subprocess.run([_nvcc(), "-O2", "-std=c++17", "-I", INC, SRC, "-o", exe], capture_output=True, text=True)
    except FileNotFoundError:
        pytest.skip("nvcc not available")
    if r.returncode != 0:
        pytest.fail("host build of the product check failed:\n" + r.stdout + r.stderr)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    vals = {}
    for line in out.splitlines():
        name, mx, rms = line.split()
        vals[name] = (float(mx), float(rms))
    print(vals)
    return vals


def test_fixed_grid_product(measured):
    mx, rms = measured["grid"]
    assert rms < 2.0 ** -41.5 and mx < 2.0 ** -35.5
    mx, rms = measured["grid_acc"]
    assert rms < 2.0 ** -41.5 and mx < 2.0 ** -35.5


def test_twosum_product(measured):
    mx, rms = measured["twosum"]
    assert rms < 2.0 ** -47.5 and mx < 2.0 ** -43.5


def test_raw_grid_pair_as_operand(measured):
    """A product's raw (unnormalised) result used as the next product's
    operand costs at most a few times the grid product's own error."""
    mx, rms = measured["grid_raw_operand"]
    assert rms < 2.0 ** -40.5
